"""Many independent scenes stepped together (ppf_multi_* in ppf_gb300_ext.h).

One solver per scene, each with its own stream, device buffers and
Newton-iteration graph, stepped by a pool of host threads inside the library,
so the scenes' launches overlap on the device. The reference has no
counterpart (its backend holds one scene per process); this is the batched
workload of many small, uneven scenes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .session import Scene, SolverError


def _declare(lib):
    P = C.c_void_p
    lib.ppf_multi_create.restype = P
    lib.ppf_multi_create.argtypes = [C.c_uint, C.POINTER(P), C.POINTER(P), C.c_uint]
    lib.ppf_multi_advance.restype = C.c_int
    lib.ppf_multi_advance.argtypes = [P, C.POINTER(abi.StepResult)]
    lib.ppf_multi_update_constraint.argtypes = [P, C.c_uint, P]
    lib.ppf_multi_fetch.argtypes = [P, C.c_uint]
    lib.ppf_multi_step_stats.argtypes = [P, C.c_uint, C.POINTER(abi.StepStats)]
    lib.ppf_multi_pcg_team.argtypes = [P, C.c_uint]
    lib.ppf_multi_set_pcg_team.argtypes = [P, C.c_uint, C.c_int]
    lib.ppf_multi_set_pcg_cta_threads.argtypes = [P, C.c_uint, C.c_uint]
    lib.ppf_multi_destroy.argtypes = [P]


class MultiSession:
    """Built scenes stepped together: step() advances every scene by one time
    step; positions(i) and stats(i) read scene i."""

    def __init__(self, scenes: list[Scene], threads: int = 32, pin_motions=None):
        """`pin_motions`: None, or per scene None or the pin motion its
        builder returned (as Session takes it)."""
        if not scenes or not all(sc.built for sc in scenes):
            raise ValueError("build the scenes first")
        self.scenes = list(scenes)
        self.pin_motions = list(pin_motions) if pin_motions else [None] * len(self.scenes)
        if len(self.pin_motions) != len(self.scenes):
            raise ValueError("one pin motion (or None) per scene")
        self.lib = self.scenes[0].lib
        _declare(self.lib)
        n = len(self.scenes)
        ds = (C.c_void_p * n)(*[sc.dataset.value for sc in self.scenes])
        pr = (C.c_void_p * n)(*[C.cast(sc.param, C.c_void_p).value for sc in self.scenes])
        self.h = self.lib.ppf_multi_create(n, ds, pr, int(threads))
        if not self.h:
            raise SolverError(self._fatal("ppf_multi_create"))
        self.results = (abi.StepResult * n)()

    def _fatal(self, what: str) -> str:
        code = int(self.lib.ppf_fatal_code())
        detail = (self.lib.ppf_fatal_detail() or b"").decode(errors="replace")
        return f"{what} failed (fatal code {code}): {detail}"

    def __len__(self) -> int:
        return len(self.scenes)

    def step(self) -> list[abi.StepResult]:
        for i, motion in enumerate(self.pin_motions):
            if motion is None:
                continue
            sc = self.scenes[i]
            prm = sc.param.contents
            pos, delta = motion(float(prm.time) + prm.dt, prm.dt)
            sc.set_pin_targets(pos, delta)
            if self.lib.ppf_multi_update_constraint(self.h, i, sc.constraint) != 0:
                raise SolverError(self._fatal("ppf_multi_update_constraint"))
        if self.lib.ppf_multi_advance(self.h, self.results) != 0:
            raise SolverError(self._fatal("ppf_multi_advance"))
        return list(self.results)

    def positions(self, i: int) -> np.ndarray:
        if self.lib.ppf_multi_fetch(self.h, int(i)) != 0:
            raise SolverError(self._fatal("ppf_multi_fetch"))
        return self.scenes[i].positions()[0]

    def stats(self, i: int) -> abi.StepStats:
        s = abi.StepStats()
        self.lib.ppf_multi_step_stats(self.h, int(i), C.byref(s))
        return s

    def pcg_team(self, i: int) -> int:
        return int(self.lib.ppf_multi_pcg_team(self.h, int(i)))

    def set_pcg_team(self, i: int, ctas: int) -> None:
        """As ppf_set_pcg_team for scene i (-1 automatic, 0 the whole grid,
        2 to 16 one cluster)."""
        if self.lib.ppf_multi_set_pcg_team(self.h, int(i), int(ctas)) != 0:
            raise ValueError(f"PCG team {ctas} is not available")

    def set_pcg_cta_threads(self, i: int, threads: int) -> None:
        """Threads per CTA of scene i's one-cluster solves (256, 512, 1024)."""
        if self.lib.ppf_multi_set_pcg_cta_threads(self.h, int(i), int(threads)) != 0:
            raise ValueError(f"{threads} threads per CTA are not available")

    def close(self) -> None:
        if self.h:
            self.lib.ppf_multi_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_bench(count: int = 256, steps: int = 100, seed: int = 0, threads: int = 32,
              compare_steps: int = 10) -> dict:
    """The uneven drops (scenes.uneven_drops) stepped together for `steps`
    time steps from t = 0, and the first `compare_steps` of them also one
    scene after another through the single-scene solver; returns the
    figures (host wall clock around the steps; scene construction and
    initialize outside it)."""
    import time

    from . import scenes
    from .session import Session

    drops = scenes.uneven_drops(count, seed)

    def build():
        return [scenes.cloth_drop(*p)[0] for p in drops]

    def together(n_steps, failures):
        built = build()
        m = MultiSession(built, threads=threads)
        newton, pcg_iters, walls = 0, np.zeros(count, np.int64), []
        for k in range(n_steps):
            t0 = time.perf_counter()
            res = m.step()
            walls.append(time.perf_counter() - t0)
            for i in range(count):
                st = m.stats(i)
                newton += st.newton_iters
                pcg_iters[i] += st.pcg_iters_total
                if not res[i].success():
                    # a failed step leaves the scene where it was (advance()
                    # returns before it commits); it is stepped again with
                    # the others
                    failures.append({"scene": i, "step": k, "drop": list(drops[i]),
                                     "result": res[i].as_dict(),
                                     "pcg_state": int(st.last_pcg_state),
                                     "pcg_break_cause": int(st.last_break_cause)})
        teams = [m.pcg_team(i) for i in range(count)]
        m.close()
        return newton, float(np.sum(walls)), pcg_iters, teams

    failures, cmp_failures = [], []
    newton, wall, pcg_iters, teams = together(steps, failures)
    n_cmp, w_cmp, _, _ = together(compare_steps, cmp_failures)
    one_newton, one_wall, one_failed = 0, 0.0, 0
    for sc in build():
        s = Session(sc)
        for _ in range(compare_steps):
            t0 = time.perf_counter()
            ok = s.step(fetch=False).success()
            one_wall += time.perf_counter() - t0
            one_newton += s.stats().newton_iters
            one_failed += 0 if ok else 1
        del s
    verts = [d[0] * d[0] for d in drops]
    it = np.sort(pcg_iters)
    return {
        "workload": (f"{count} uneven cloth drops (sides 16-96 log-uniform, heights 0.2-1.0 m, "
                     "sphere or box colliders; seeded), each with its own solver, stepped "
                     f"together by {threads} host threads (ppf_multi_advance)"),
        "scenes": count, "vertices_total": int(sum(verts)),
        "steps": steps, "from": "t = 0",
        "newton_iters": newton, "wall_s": round(wall, 3),
        "newton_iters_per_s": round(newton / wall, 1),
        "scene_steps_per_s": round(count * steps / wall, 1),
        "pcg_iters_per_scene_median": int(it[len(it) // 2]),
        "pcg_iters_per_scene_p90": int(it[int(0.9 * (len(it) - 1))]),
        "pcg_teams": {str(t): teams.count(t) for t in sorted(set(teams))},
        "failed_scene_steps": len(failures), "failures": failures[:8],
        "first_steps": {"steps": compare_steps,
                        "together_newton_iters_per_s": round(n_cmp / w_cmp, 1),
                        "one_by_one_newton_iters_per_s": round(one_newton / one_wall, 1),
                        "speedup": round((n_cmp / w_cmp) / (one_newton / one_wall), 2),
                        "failed_scene_steps": [len(cmp_failures), one_failed]},
    }
