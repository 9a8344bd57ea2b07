"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Imported only by tests/, by __graft_entry__.smoke() and by bench.py's CPU
baseline arm, as the checker. The product (ppf_gb300 / libppf_gb300.so)
never imports, loads or calls anything here.

OracleSession mirrors ppf_gb300.session.Session on the same built Scene: it
reads the same DataSet the product's initialize() reads, and advances its own
copy of the state with the restatement in oracle_solver.cpp.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from ppf_gb300 import abi, build as _build
from ppf_gb300._lib import f32p, f32p_opt, u32p, u32p_opt

_ORACLE = None
_REF = None


def oracle() -> C.CDLL:
    global _ORACLE
    if _ORACLE is None:
        if not _build.ORACLE_LIB.exists():
            _build.build_oracle()
        lib = C.CDLL(str(_build.ORACLE_LIB))
        _declare(lib)
        _ORACLE = lib
    return _ORACLE


def reference():
    """The reference's own element math compiled from its sources
    (oracle/Makefile), or None where those sources are not available."""
    global _REF
    if _REF is None:
        path = Path(_build.REF_LIB)
        if not path.exists():
            return None
        _REF = C.CDLL(str(path))
    return _REF


_REF_PIPE = None


def reference_pipeline():
    """The reference's own assembly, contact detection, line searches and
    intersection check compiled from its sources with host shims
    (oracle/ref_pipeline.cpp), or None where those sources are not available."""
    global _REF_PIPE
    if _REF_PIPE is None:
        path = Path(_build.REF_PIPE_LIB)
        if not path.exists():
            return None
        lib = C.CDLL(str(path))
        P = C.c_void_p
        lib.refpipe_init.restype = C.c_bool
        lib.refpipe_init.argtypes = [P, C.POINTER(abi.ParamSet)]
        lib.refpipe_state.restype = None
        lib.refpipe_state.argtypes = [f32p, f32p, C.POINTER(abi.ParamSet)]
        lib.refpipe_assemble.restype = C.c_uint
        lib.refpipe_assemble.argtypes = [f32p, f32p, C.c_float]
        lib.refpipe_blocks.restype = C.c_uint
        lib.refpipe_blocks.argtypes = [u32p_opt, u32p_opt, f32p_opt]
        lib.refpipe_force.restype = None
        lib.refpipe_force.argtypes = [f32p]
        lib.refpipe_line_search.restype = C.c_float
        lib.refpipe_line_search.argtypes = [f32p, f32p, C.POINTER(C.c_uint), C.POINTER(C.c_int)]
        lib.refpipe_strain_line_search.restype = C.c_float
        lib.refpipe_strain_line_search.argtypes = [f32p, f32p]
        lib.refpipe_rod_strain_line_search.restype = C.c_float
        lib.refpipe_rod_strain_line_search.argtypes = [f32p, f32p]
        lib.refpipe_check_intersection.restype = C.c_bool
        lib.refpipe_check_intersection.argtypes = [f32p]
        _REF_PIPE = lib
    return _REF_PIPE


def _declare(lib):
    P = C.c_void_p
    lib.oracle_lbvh_build.restype = C.c_uint
    lib.oracle_lbvh_build.argtypes = [
        C.c_int, f32p, f32p, C.c_uint, u32p_opt, C.c_uint, f32p, C.c_float,
        u32p_opt, f32p_opt, u32p_opt]
    lib.oracle_stable_sort.restype = None
    lib.oracle_stable_sort.argtypes = [u32p, u32p, C.c_uint, C.c_int]
    lib.oracle_initialize.restype = C.c_bool
    lib.oracle_initialize.argtypes = [P, C.POINTER(abi.ParamSet)]
    lib.oracle_advance.restype = None
    lib.oracle_advance.argtypes = [C.POINTER(abi.StepResult)]
    lib.oracle_fetch.restype = None
    lib.oracle_fetch.argtypes = [f32p, f32p_opt]
    lib.oracle_time.restype = C.c_double
    lib.oracle_check_intersection.restype = C.c_bool
    lib.oracle_check_intersection.argtypes = [f32p]
    lib.oracle_ls_trace.restype = C.c_bool
    lib.oracle_ls_trace.argtypes = [C.c_uint, f32p, f32p, C.POINTER(C.c_float),
                                    C.POINTER(C.c_float)]
    lib.oracle_intersection_records.restype = C.c_uint
    lib.oracle_intersection_records.argtypes = [f32p, u32p, C.c_uint]
    lib.oracle_update_constraint.argtypes = [P]
    lib.oracle_step_stats.argtypes = [C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                      C.POINTER(C.c_float)]
    lib.oracle_newton_system.restype = C.c_int
    lib.oracle_newton_system.argtypes = [f32p, C.POINTER(C.c_uint), C.POINTER(C.c_float)]
    lib.oracle_system_sizes.argtypes = [u32p]
    lib.oracle_assemble_first.restype = C.c_float
    lib.oracle_assemble_first.argtypes = [C.c_int, f32p_opt]
    lib.oracle_param.restype = None
    lib.oracle_param.argtypes = [C.POINTER(abi.ParamSet)]
    lib.oracle_line_search_at.restype = C.c_float
    lib.oracle_line_search_at.argtypes = [f32p, f32p, C.POINTER(C.c_uint), C.POINTER(C.c_int)]
    lib.oracle_strain_line_search_at.restype = C.c_float
    lib.oracle_strain_line_search_at.argtypes = [f32p, f32p]
    lib.oracle_system.argtypes = [u32p_opt, u32p_opt, f32p_opt, u32p_opt, u32p_opt, f32p_opt,
                                  f32p_opt, f32p_opt, u32p_opt, u32p_opt, u32p_opt, u32p_opt]


class OracleSession:
    """The oracle's step loop on a built ppf_gb300.session.Scene."""

    def __init__(self, scene, pin_motion=None, param=None):
        self.lib = oracle()
        self.scene = scene
        self.pin_motion = pin_motion
        self.n = scene.vertex_count
        # the oracle keeps its own copy of the ParamSet
        self.param = abi.ParamSet.from_buffer_copy(param if param is not None
                                                   else scene.param.contents)
        if not self.lib.oracle_initialize(scene.dataset, C.byref(self.param)):
            raise RuntimeError("oracle: the scene starts self-intersecting")

    @property
    def time(self) -> float:
        return float(self.lib.oracle_time())

    def step(self) -> abi.StepResult:
        if self.pin_motion is not None:
            pos, delta = self.pin_motion(self.time + self.param.dt, self.param.dt)
            self.scene.set_pin_targets(pos, delta)
            self.lib.oracle_update_constraint(self.scene.constraint)
        res = abi.StepResult()
        self.lib.oracle_advance(C.byref(res))
        return res

    def positions(self):
        curr = np.empty(3 * self.n, np.float32)
        prev = np.empty(3 * self.n, np.float32)
        self.lib.oracle_fetch(curr, prev)
        return curr.reshape(-1, 3), prev.reshape(-1, 3)

    def intersection_free(self, x) -> bool:
        """Independent intersection check of positions x (e.g. the GPU's)."""
        return bool(self.lib.oracle_check_intersection(
            np.ascontiguousarray(x, np.float32).reshape(-1)))

    def intersection_records(self, x, max_count: int = 4096):
        """Every intersecting pair of positions x as an array of (type, elem0,
        elem1) rows, in the reference's record types (0 face-edge, 1
        edge-edge, 2 collision face-edge)."""
        out = np.zeros(3 * max_count, np.uint32)
        n = self.lib.oracle_intersection_records(
            np.ascontiguousarray(x, np.float32).reshape(-1), out, max_count)
        return out[:3 * min(n, max_count)].reshape(-1, 3), int(n)

    def ls_trace(self, k: int = 0):
        """Line-search inputs of the k-th newest Newton iteration: (x0, x1,
        contact toi, raw strain-limit toi), or None."""
        x0 = np.empty(3 * self.n, np.float32)
        x1 = np.empty(3 * self.n, np.float32)
        tc, ts = C.c_float(), C.c_float()
        if not self.lib.oracle_ls_trace(k, x0, x1, C.byref(tc), C.byref(ts)):
            return None
        return x0, x1, tc.value, ts.value

    def stats(self):
        a, b, c = C.c_uint(), C.c_uint(), C.c_float()
        self.lib.oracle_step_stats(C.byref(a), C.byref(b), C.byref(c))
        return {"newton_iters": a.value, "pcg_iters_total": b.value, "step_ms": c.value}

    def newton_system(self):
        """First Newton system of a step at the current state: (state, dx,
        iters, reresid) and the kept system (see system())."""
        dx = np.empty(3 * self.n, np.float32)
        it, rr = C.c_uint(), C.c_float()
        st = self.lib.oracle_newton_system(dx, C.byref(it), C.byref(rr))
        return st, dx.reshape(-1, 3), it.value, rr.value

    def system(self):
        sizes = np.zeros(6, np.uint32)
        self.lib.oracle_system_sizes(sizes)
        return _system(self.lib.oracle_system, self.n, sizes)


def _system(fn, n, sizes):
    nf, nd, npf, npe, npp, nee = (int(x) for x in sizes)
    out = {
        "f_off": np.zeros(n + 1, np.uint32), "f_col": np.zeros(max(nf, 1), np.uint32),
        "f_val": np.zeros(9 * max(nf, 1), np.float32),
        "d_off": np.zeros(n + 1, np.uint32), "d_col": np.zeros(max(nd, 1), np.uint32),
        "d_val": np.zeros(9 * max(nd, 1), np.float32),
        "diag": np.zeros(9 * n, np.float32), "force": np.zeros(3 * n, np.float32),
        "pf": np.zeros(2 * max(npf, 1), np.uint32), "pe": np.zeros(3 * max(npe, 1), np.uint32),
        "pp": np.zeros(3 * max(npp, 1), np.uint32), "ee": np.zeros(2 * max(nee, 1), np.uint32),
    }
    fn(out["f_off"], out["f_col"], out["f_val"], out["d_off"], out["d_col"], out["d_val"],
       out["diag"], out["force"], out["pf"], out["pe"], out["pp"], out["ee"])
    out["f_col"] = out["f_col"][:nf]
    out["f_val"] = out["f_val"][:9 * nf].reshape(-1, 9)
    out["d_col"] = out["d_col"][:nd]
    out["d_val"] = out["d_val"][:9 * nd].reshape(-1, 9)
    out["diag"] = out["diag"].reshape(-1, 9)
    out["force"] = out["force"].reshape(-1, 3)
    out["pf"] = out["pf"][:2 * npf].reshape(-1, 2)
    out["pe"] = out["pe"][:3 * npe].reshape(-1, 3)
    out["pp"] = out["pp"][:3 * npp].reshape(-1, 3)
    out["ee"] = out["ee"][:2 * nee].reshape(-1, 2)
    return out


def product_system(lib, n):
    """The system kept by the product's ppf_debug_newton_system, in the same
    layout as OracleSession.system()."""
    sizes = np.zeros(6, np.uint32)
    lib.ppf_debug_system_sizes(sizes)
    lib.ppf_debug_system.argtypes = [u32p_opt, u32p_opt, f32p_opt, u32p_opt, u32p_opt,
                                     f32p_opt, f32p_opt, f32p_opt, u32p_opt, u32p_opt,
                                     u32p_opt, u32p_opt]
    return _system(lib.ppf_debug_system, n, sizes)
