"""ctypes mirrors of the C ABI structs a host touches directly.

ParamSet and StepResult are the reference's (crates/ppf-cts-solver/src/cpp/
data.hpp:515-595, bound on the Rust side by crates/ppf-cts-solver/src/
data.rs); ShellMaterial and StepStats belong to this library's own headers
(include/ppf_gb300_scene.h, include/ppf_gb300_ext.h). The byte layout of each
is checked against the C headers by tests/test_abi_layout.py.
"""
from __future__ import annotations

import ctypes as C

STATS_MAX_SOLVES = 256

BARRIER_CUBIC, BARRIER_QUAD, BARRIER_LOG = 0, 1, 2
PRECOND_BLOCK_JACOBI, PRECOND_FIRST_ORDER, PRECOND_LEARNED = 0, 1, 2
PRECOND_FSAI = 4
FRICTION_MIN, FRICTION_MAX, FRICTION_MEAN = 0, 1, 2
MODEL_ARAP, MODEL_STVK, MODEL_BARAFF_WITKIN, MODEL_SNHK = 0, 1, 2, 3


class Vec3f(C.Structure):
    _fields_ = [("v", C.c_float * 3)]


class ParamSet(C.Structure):
    _fields_ = [
        ("time", C.c_double),
        ("air_friction", C.c_float),
        ("air_density", C.c_float),
        ("constraint_tol", C.c_float),
        ("prev_dt", C.c_float),
        ("dt", C.c_float),
        ("playback", C.c_float),
        ("min_newton_steps", C.c_uint),
        ("target_toi", C.c_float),
        ("stitch_length_factor", C.c_float),
        ("cg_max_iter", C.c_uint),
        ("cg_tol", C.c_float),
        ("line_search_max_t", C.c_float),
        ("ccd_eps", C.c_float),
        ("max_dx", C.c_float),
        ("eiganalysis_eps", C.c_float),
        ("friction_eps", C.c_float),
        ("isotropic_air_friction", C.c_float),
        ("gravity", Vec3f),
        ("wind", Vec3f),
        ("barrier", C.c_int),
        ("friction_mode", C.c_int),
        ("csrmat_max_nnz", C.c_uint),
        ("fix_xz", C.c_float),
        ("disable_contact", C.c_bool),
        ("inactive_momentum", C.c_bool),
        ("precond", C.c_int),
        ("schwarz_levels", C.c_uint),
        ("max_newton_steps", C.c_uint),
        ("disable_pin_dof_removal", C.c_bool),
    ]


class StepResult(C.Structure):
    _fields_ = [
        ("time", C.c_double),
        ("ccd_success", C.c_bool),
        ("pcg_success", C.c_bool),
        ("intersection_free", C.c_bool),
        ("newton_progress", C.c_bool),
        ("pin_feasible", C.c_bool),
        ("contact_separated", C.c_bool),
    ]

    def success(self) -> bool:
        """The reference's StepResult::success (data.hpp:584-588)."""
        return bool(self.ccd_success and self.pcg_success and self.intersection_free
                    and self.newton_progress and self.pin_feasible
                    and self.contact_separated)

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ShellMaterial(C.Structure):
    _fields_ = [
        ("model", C.c_int),
        ("density", C.c_float),
        ("young_mod", C.c_float),
        ("poiss_rat", C.c_float),
        ("bend", C.c_float),
        ("strain_limit", C.c_float),
        ("contact_gap", C.c_float),
        ("contact_offset", C.c_float),
        ("friction", C.c_float),
        ("deform_damping", C.c_float),
        ("bend_damping", C.c_float),
    ]


class SolidMaterial(C.Structure):
    _fields_ = [
        ("model", C.c_int),
        ("density", C.c_float),
        ("young_mod", C.c_float),
        ("poiss_rat", C.c_float),
        ("contact_gap", C.c_float),
        ("contact_offset", C.c_float),
        ("friction", C.c_float),
        ("deform_damping", C.c_float),
    ]


class RodMaterial(C.Structure):
    _fields_ = [
        ("density", C.c_float),
        ("young_mod", C.c_float),
        ("bend", C.c_float),
        ("length_factor", C.c_float),
        ("strain_limit", C.c_float),
        ("contact_gap", C.c_float),
        ("contact_offset", C.c_float),
        ("friction", C.c_float),
        ("deform_damping", C.c_float),
        ("bend_damping", C.c_float),
        ("bend_rest_from_geometry", C.c_int),
    ]


class StepStats(C.Structure):
    _fields_ = [
        ("newton_iters", C.c_uint),
        ("pcg_iters_total", C.c_uint),
        ("pcg_solves", C.c_uint),
        ("pcg_ms_total", C.c_float),
        ("step_ms", C.c_float),
        ("max_contacts", C.c_uint),
        ("max_dyn_blocks", C.c_uint),
        ("pcg_ms", C.c_float * STATS_MAX_SOLVES),
        ("pcg_iters", C.c_uint * STATS_MAX_SOLVES),
        ("toi", C.c_float * STATS_MAX_SOLVES),
        ("fixed_blocks", C.c_uint),
        ("vertices", C.c_uint),
        ("dyn_blocks", C.c_uint * STATS_MAX_SOLVES),
        ("precond_kind", C.c_uint),
        ("fallbacks", C.c_uint),
        ("factor_iters_total", C.c_uint),
        ("last_pcg_state", C.c_int),
        ("last_break_cause", C.c_int),
        ("last_pcg_resid", C.c_float),
        ("last_break_val", C.c_float),
    ]


class IntersectionRecord(C.Structure):
    _fields_ = [
        ("type", C.c_uint),
        ("elem0", C.c_uint),
        ("elem1", C.c_uint),
        ("num_verts0", C.c_uint),
        ("num_verts1", C.c_uint),
        ("positions", C.c_float * 15),
    ]


# struct name in the C headers -> ctypes mirror
MIRRORS = {
    "PpfParamSet": ParamSet,
    "PpfStepResult": StepResult,
    "PpfShellMaterial": ShellMaterial,
    "PpfStepStats": StepStats,
    "PpfIntersectionRecord": IntersectionRecord,
}
