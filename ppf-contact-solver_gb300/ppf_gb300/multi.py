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
    lib.ppf_multi_destroy.argtypes = [P]


class MultiSession:
    """Built scenes stepped together: step() advances every scene by one time
    step; positions(i) and stats(i) read scene i."""

    def __init__(self, scenes: list[Scene], threads: int = 16):
        if not scenes or not all(sc.built for sc in scenes):
            raise ValueError("build the scenes first")
        self.scenes = list(scenes)
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

    def close(self) -> None:
        if self.h:
            self.lib.ppf_multi_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
