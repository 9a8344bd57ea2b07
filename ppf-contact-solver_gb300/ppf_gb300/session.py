"""Host-side scene building and the per-step session over the C ABI.

`Scene` wraps the C++ scene builder of libppf_gb300.so (include/
ppf_gb300_scene.h), which produces the DataSet / ParamSet / Constraint the
reference's Rust driver hands to its backend (crates/ppf-cts-solver/src/
builder.rs build(), make_param()). `Session` drives the reference's step
entry points on that DataSet exactly as the Rust driver does
(crates/ppf-cts-solver/src/backend.rs:626-1030): initialize once, then per
step update_constraint (when pins move), advance, fetch.

Nothing here computes physics: every step goes through the CUDA library, and
a missing library raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from ._lib import product

_f32 = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_u32 = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_declared = set()


def _declare(lib):
    if id(lib) in _declared:
        return
    P = C.c_void_p
    lib.ppf_scene_create.restype = P
    lib.ppf_scene_create.argtypes = []
    lib.ppf_scene_destroy.argtypes = [P]
    lib.ppf_scene_default_param.argtypes = [C.POINTER(abi.ParamSet)]
    lib.ppf_scene_add_shell.restype = C.c_uint
    lib.ppf_scene_add_shell.argtypes = [P, _f32, C.c_uint, _u32, C.c_uint,
                                        C.POINTER(abi.ShellMaterial)]
    lib.ppf_scene_add_rod.restype = C.c_uint
    lib.ppf_scene_add_rod.argtypes = [P, _f32, C.c_uint, _u32, C.c_uint,
                                      C.POINTER(abi.RodMaterial)]
    lib.ppf_scene_add_solid.restype = C.c_uint
    lib.ppf_scene_add_solid.argtypes = [P, _f32, C.c_uint, _u32, C.c_uint,
                                        C.POINTER(abi.SolidMaterial)]
    lib.ppf_scene_add_stitch.restype = C.c_int
    lib.ppf_scene_add_stitch.argtypes = [P, _u32, _f32, C.c_float]
    lib.ppf_scene_set_velocity.argtypes = [P, _f32]
    lib.ppf_scene_pin.argtypes = [P, _u32, C.c_uint, C.c_int]
    lib.ppf_scene_pull.argtypes = [P, _u32, C.c_uint, C.c_float]
    lib.ppf_scene_add_sphere.argtypes = [P, _f32, C.c_float, C.c_float, C.c_float,
                                         C.c_int, C.c_int]
    lib.ppf_scene_add_floor.argtypes = [P, _f32, _f32, C.c_float, C.c_float]
    lib.ppf_scene_add_collision_mesh.argtypes = [P, _f32, C.c_uint, _u32, C.c_uint, C.c_float,
                                                 C.c_float, C.c_float]
    lib.ppf_scene_build.restype = C.c_int
    lib.ppf_scene_build.argtypes = [P, C.POINTER(abi.ParamSet)]
    lib.ppf_scene_dataset.restype = P
    lib.ppf_scene_dataset.argtypes = [P]
    lib.ppf_scene_param.restype = C.POINTER(abi.ParamSet)
    lib.ppf_scene_param.argtypes = [P]
    lib.ppf_scene_constraint.restype = P
    lib.ppf_scene_constraint.argtypes = [P]
    lib.ppf_scene_set_pin_targets.argtypes = [P, _f32, C.c_void_p]
    lib.ppf_scene_vertex_count.restype = C.c_uint
    lib.ppf_scene_vertex_count.argtypes = [P]
    lib.ppf_scene_positions.argtypes = [P, C.c_void_p, C.c_void_p]
    lib.ppf_scene_set_positions.argtypes = [P, C.c_void_p, C.c_void_p]
    lib.ppf_scene_array.restype = C.c_size_t
    lib.ppf_scene_array.argtypes = [P, C.c_char_p, C.c_void_p]
    lib.ppf_set_preconditioner.restype = C.c_int
    lib.ppf_set_preconditioner.argtypes = [C.c_int, C.c_float]
    # reference entry points (include/ppf_gb300.h)
    lib.initialize.restype = C.c_bool
    lib.initialize.argtypes = [P, C.POINTER(abi.ParamSet)]
    lib.advance.restype = None
    lib.advance.argtypes = [C.POINTER(abi.StepResult)]
    lib.fetch.restype = None
    lib.fetch.argtypes = []
    lib.update_constraint.restype = None
    lib.update_constraint.argtypes = [P]
    lib.gather_current_positions.argtypes = [_u32, C.c_uint, _f32]
    lib.override_velocity.argtypes = [_u32, C.c_uint, C.c_float, C.c_float, C.c_float,
                                      C.c_float]
    lib.fetch_intersection_records.restype = C.c_uint
    lib.fetch_intersection_records.argtypes = [C.POINTER(abi.IntersectionRecord), C.c_uint]
    lib.ppf_fatal_code.restype = C.c_ubyte
    lib.ppf_fatal_detail.restype = C.c_char_p
    lib.ppf_step_stats.argtypes = [C.POINTER(abi.StepStats)]
    lib.ppf_stream.restype = C.c_void_p
    lib.ppf_stream.argtypes = []
    lib.ppf_kernel_launches.restype = C.c_ulonglong
    lib.ppf_kernel_launches.argtypes = []
    lib.ppf_debug_newton_system.restype = C.c_int
    lib.ppf_debug_newton_system.argtypes = [_f32, C.POINTER(C.c_uint), C.POINTER(C.c_float)]
    lib.ppf_debug_system_sizes.argtypes = [_u32]
    _declared.add(id(lib))


def default_param(dt: float = 1e-3) -> abi.ParamSet:
    """The reference's ParamSet defaults (builder.rs make_param) at step dt."""
    lib = product()
    _declare(lib)
    p = abi.ParamSet()
    lib.ppf_scene_default_param(C.byref(p))
    p.dt = dt
    p.prev_dt = dt
    return p


@dataclass
class Material:
    """Shell material in the reference's units (params.rs object_param):
    young_mod is Young's modulus divided by density (Pa / (kg/m^2))."""

    density: float = 1.0
    young_mod: float = 1000.0
    poiss_rat: float = 0.35
    bend: float = 10.0
    strain_limit: float = 0.0
    contact_gap: float = 1e-3
    contact_offset: float = 0.0
    friction: float = 0.0
    model: int = abi.MODEL_BARAFF_WITKIN
    deform_damping: float = 0.0
    bend_damping: float = 0.0

    def to_c(self) -> abi.ShellMaterial:
        return abi.ShellMaterial(self.model, self.density, self.young_mod, self.poiss_rat,
                                 self.bend, self.strain_limit, self.contact_gap,
                                 self.contact_offset, self.friction, self.deform_damping,
                                 self.bend_damping)


@dataclass
class SolidMaterial:
    """Solid (tet) material in the reference's units (scene.rs tet
    parameters): density in kg/m^3, young_mod pre-divided by density."""

    density: float = 1000.0
    young_mod: float = 500.0
    poiss_rat: float = 0.35
    model: int = abi.MODEL_ARAP
    contact_gap: float = 1e-3
    contact_offset: float = 0.0
    friction: float = 0.0
    deform_damping: float = 0.0

    def to_c(self) -> abi.SolidMaterial:
        return abi.SolidMaterial(self.model, self.density, self.young_mod, self.poiss_rat,
                                 self.contact_gap, self.contact_offset, self.friction,
                                 self.deform_damping)


@dataclass
class RodMaterial:
    """Rod material in the reference's units (scene.rs rod parameters):
    density in kg/m, young_mod the stretch stiffness per unit edge mass."""

    density: float = 1.0
    young_mod: float = 1000.0
    bend: float = 0.0
    length_factor: float = 1.0
    strain_limit: float = 0.0
    contact_gap: float = 1e-3
    contact_offset: float = 0.0
    friction: float = 0.0
    deform_damping: float = 0.0
    bend_damping: float = 0.0
    bend_rest_from_geometry: bool = False

    def to_c(self) -> abi.RodMaterial:
        return abi.RodMaterial(self.density, self.young_mod, self.bend, self.length_factor,
                               self.strain_limit, self.contact_gap, self.contact_offset,
                               self.friction, self.deform_damping, self.bend_damping,
                               1 if self.bend_rest_from_geometry else 0)


class Scene:
    """A scene under construction, then the built DataSet that owns the host
    arrays initialize() reads and fetch() writes."""

    def __init__(self):
        self.lib = product()
        _declare(self.lib)
        self.h = C.c_void_p(self.lib.ppf_scene_create())
        self.n_pins = 0
        self.n_spheres = 0
        self.n_floors = 0
        self.n_collision_vertices = 0
        self._rod_count = 0
        self._rod_mats = []
        self._vert_inputs = []
        self._solids = []
        self.built = False

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            self.lib.ppf_scene_destroy(h)
            self.h = C.c_void_p(0)

    def add_shell(self, vertices, faces, material: Material) -> int:
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1)
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1)
        m = material.to_c()
        self._vert_inputs.append(v.reshape(-1, 3).copy())
        return int(self.lib.ppf_scene_add_shell(self.h, v, v.size // 3, f, f.size // 3,
                                                C.byref(m)))

    def add_rod(self, vertices, edges, material: RodMaterial) -> int:
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1)
        e = np.ascontiguousarray(edges, np.uint32).reshape(-1)
        m = material.to_c()
        self._rod_count += e.size // 2
        self._rod_mats.extend([material] * (e.size // 2))
        self._vert_inputs.append(v.reshape(-1, 3).copy())
        return int(self.lib.ppf_scene_add_rod(self.h, v, v.size // 3, e, e.size // 2,
                                              C.byref(m)))

    def add_solid(self, vertices, tets, material: SolidMaterial) -> int:
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1)
        t = np.ascontiguousarray(tets, np.uint32).reshape(-1)
        m = material.to_c()
        self._vert_inputs.append(v.reshape(-1, 3).copy())
        self._solids.append((len(np.concatenate(self._vert_inputs)) - v.size // 3,
                             t.reshape(-1, 4).copy(), material))
        return int(self.lib.ppf_scene_add_solid(self.h, v, v.size // 3, t, t.size // 4,
                                                C.byref(m)))

    def add_stitch(self, index, weight, stiffness: float = 1.0) -> None:
        """A stitch between the barycentric points index[0:3] / weight[0:3]
        and index[3:6] / weight[3:6] (vertex indices as added)."""
        i = np.ascontiguousarray(index, np.uint32).reshape(6)
        w = np.ascontiguousarray(weight, np.float32).reshape(6)
        if self.lib.ppf_scene_add_stitch(self.h, i, w, float(stiffness)) != 0:
            raise ValueError("stitch index out of range")

    def set_velocity(self, velocity):
        v = np.ascontiguousarray(velocity, np.float32).reshape(-1)
        assert v.size == 3 * self.vertex_count
        self.lib.ppf_scene_set_velocity(self.h, v)

    def pin(self, indices, kinematic: bool = False):
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        self.lib.ppf_scene_pin(self.h, idx, idx.size, 1 if kinematic else 0)
        self.n_pins += idx.size

    def pull(self, indices, weight: float):
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        self.lib.ppf_scene_pull(self.h, idx, idx.size, weight)

    def add_sphere(self, center, radius, contact_gap=1e-3, friction=0.0, reverse=False,
                   bowl=False):
        c = np.ascontiguousarray(center, np.float32)
        self.lib.ppf_scene_add_sphere(self.h, c, radius, contact_gap, friction,
                                      int(reverse), int(bowl))
        self.n_spheres += 1

    def add_floor(self, ground, up=(0.0, 1.0, 0.0), contact_gap=1e-3, friction=0.0):
        self.lib.ppf_scene_add_floor(self.h, np.ascontiguousarray(ground, np.float32),
                                     np.ascontiguousarray(up, np.float32), contact_gap,
                                     friction)
        self.n_floors += 1

    def add_collision_mesh(self, vertices, faces, contact_gap=1e-3, contact_offset=0.0,
                           friction=0.0):
        """A static triangle mesh that the cloth collides with but that has no
        degrees of freedom (the reference's Constraint::mesh)."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1)
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1)
        self.lib.ppf_scene_add_collision_mesh(self.h, v, v.size // 3, f, f.size // 3,
                                              contact_gap, contact_offset, friction)
        self.n_collision_vertices += v.size // 3

    @property
    def _rest_positions(self) -> np.ndarray:
        """The vertex positions the objects were added with (the builder's
        rest shape), in vertex order."""
        return np.concatenate(self._vert_inputs) if self._vert_inputs else np.zeros((0, 3))

    @property
    def vertex_count(self) -> int:
        return int(self.lib.ppf_scene_vertex_count(self.h))

    def build(self, param: abi.ParamSet) -> "Scene":
        rc = self.lib.ppf_scene_build(self.h, C.byref(param))
        if rc != 0:
            raise ValueError(f"scene build failed ({rc}): degenerate triangle")
        self.built = True
        return self

    @property
    def dataset(self) -> C.c_void_p:
        return C.c_void_p(self.lib.ppf_scene_dataset(self.h))

    @property
    def param(self):
        """Pointer to the ParamSet initialize() keeps; advance() updates its
        time and prev_dt in place."""
        return self.lib.ppf_scene_param(self.h)

    @property
    def constraint(self) -> C.c_void_p:
        return C.c_void_p(self.lib.ppf_scene_constraint(self.h))

    def positions(self):
        n = self.vertex_count
        curr = np.empty((n, 3), np.float32)
        prev = np.empty((n, 3), np.float32)
        self.lib.ppf_scene_positions(self.h, curr.ctypes.data_as(C.c_void_p),
                                     prev.ctypes.data_as(C.c_void_p))
        return curr, prev

    def set_positions(self, curr=None, prev=None):
        n = self.vertex_count
        args = []
        keep = []
        for a in (curr, prev):
            if a is None:
                args.append(None)
            else:
                a = np.ascontiguousarray(a, np.float32).reshape(n, 3)
                keep.append(a)
                args.append(a.ctypes.data_as(C.c_void_p))
        self.lib.ppf_scene_set_positions(self.h, *args)

    _ARRAY_DTYPES = {"inv_rest2x2": np.float32, "vertex_mass": np.float32,
                     "vertex_area": np.float32, "face_area": np.float32,
                     "face_mass": np.float32, "edge_length": np.float32,
                     "hinge_length": np.float32, "hinge_area": np.float32,
                     "face_mu": np.float32, "face_lambda": np.float32,
                     "hinge_bend": np.float32, "edge_initial_length": np.float32,
                     "edge_mass": np.float32, "edge_stiffness": np.float32,
                     "edge_bend": np.float32, "rest_bend_angle": np.float32,
                     "vertex_ghat": np.float32, "vertex_offset": np.float32,
                     "vertex_friction": np.float32, "inv_rest3x3": np.float32,
                     "tet_mass": np.float32, "tet_volume": np.float32,
                     "vertex_volume": np.float32, "face_type": np.uint8,
                     "hinge_type": np.uint8}

    def array(self, name: str) -> np.ndarray:
        """A named array of the built DataSet (ppf_scene_array): topology
        (face, edge, hinge), inv_rest2x2, the fixed pattern and its transpose
        and slot tables, or a per-element float (vertex_mass, face_area, ...)."""
        dtype = self._ARRAY_DTYPES.get(name, np.uint32)
        nbytes = int(self.lib.ppf_scene_array(self.h, name.encode(), None))
        if nbytes == C.c_size_t(-1).value:
            raise KeyError(name)
        out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype)
        if nbytes:
            self.lib.ppf_scene_array(self.h, name.encode(), out.ctypes.data_as(C.c_void_p))
        return out

    def set_pin_targets(self, position, step_delta=None):
        pos = np.ascontiguousarray(position, np.float32).reshape(-1)
        assert pos.size == 3 * self.n_pins
        if step_delta is None:
            self.lib.ppf_scene_set_pin_targets(self.h, pos, None)
        else:
            d = np.ascontiguousarray(step_delta, np.float32).reshape(-1)
            self.lib.ppf_scene_set_pin_targets(self.h, pos, d.ctypes.data_as(C.c_void_p))


class SolverError(RuntimeError):
    pass


class Session:
    """The reference's per-step driver over one built scene: initialize(),
    then step() = [update_constraint()] + advance() + fetch().

    Only one Session may be live per process: the library, like the
    reference's backend, keeps its state in process-wide singletons."""

    def __init__(self, scene: Scene, pin_motion=None):
        if not scene.built:
            raise ValueError("build the scene first")
        self.scene = scene
        self.lib = scene.lib
        self.pin_motion = pin_motion
        self.frame = 0
        ok = self.lib.initialize(scene.dataset, scene.param)
        if not ok:
            code = int(self.lib.ppf_fatal_code())
            detail = (self.lib.ppf_fatal_detail() or b"").decode(errors="replace")
            raise SolverError(f"initialize failed (fatal code {code}): {detail}")

    @property
    def param(self) -> abi.ParamSet:
        return self.scene.param.contents

    @property
    def time(self) -> float:
        return float(self.param.time)

    def step(self, fetch: bool = True) -> abi.StepResult:
        if self.pin_motion is not None:
            pos, delta = self.pin_motion(self.time + self.param.dt, self.param.dt)
            self.scene.set_pin_targets(pos, delta)
            self.lib.update_constraint(self.scene.constraint)
        res = abi.StepResult()
        self.lib.advance(C.byref(res))
        code = int(self.lib.ppf_fatal_code())
        if code:
            detail = (self.lib.ppf_fatal_detail() or b"").decode(errors="replace")
            raise SolverError(f"advance failed (fatal code {code}): {detail}")
        if fetch:
            self.lib.fetch()
        self.frame += 1
        return res

    def positions(self):
        return self.scene.positions()[0]

    def stats(self) -> abi.StepStats:
        s = abi.StepStats()
        self.lib.ppf_step_stats(C.byref(s))
        return s

    def set_preconditioner(self, kind: int, param: float = 0.0) -> None:
        """abi.PRECOND_BLOCK_JACOBI (the reference's), PRECOND_FIRST_ORDER
        (param: the factor's coupling weight, 0.5 by default) or
        PRECOND_LEARNED (after the network's weights are loaded)."""
        if self.lib.ppf_set_preconditioner(int(kind), float(param)) != 0:
            raise ValueError(f"preconditioner kind {kind} is not available")

    def intersection_records(self, max_count: int = 256):
        buf = (abi.IntersectionRecord * max_count)()
        n = self.lib.fetch_intersection_records(buf, max_count)
        return list(buf[:n])
