"""Seeded synthetic workloads of the per-step contact solve.

Each builder returns a built `Scene` plus the pin motion (or None) a
`Session` needs. The reference solver is Y-up (gravity (0, -9.8, 0)), so a
height is +y and "rotation about z" of a sheet lying in the XZ plane is taken
about the vertical axis y. Young's modulus is given in Pa and divided by the
areal density, as the reference's `young-mod` parameter expects
(crates/ppf-cts-core/src/datamodel/params.rs, "young-mod").

Workloads (sizes as named by the benchmark):
  cloth_sphere    one 64x64 sheet (1 m) at y = 1 over a fixed sphere r 0.3
  stacked_sheets  8 sheets of 128x128, seeded rotation / offsets, 2 cm apart
                  above a fixed 0.6 m cube (a fully pinned triangle shell)
  twisted_tube    tube r 0.1, L 1, 256 around x 512 along, end rings pinned
                  and spun at +-2 rad/s about the tube axis
  sphere_field    1024x1024 sheet over 50 seeded fixed spheres
Any builder takes a `scale` (vertices per side divided by it) so tests can
run the same scene family at a size the oracle finishes in seconds.
"""
from __future__ import annotations

import math

import numpy as np

from . import meshes
from .session import Material, Scene, default_param

E_PA = 1e4
DENSITY = 0.2


def cloth_material() -> Material:
    """Baraff-Witkin shell shared by the workloads: density 0.2 kg/m^2,
    Young 1e4 Pa, Poisson 0.25, contact gap 1e-3 m, friction 0.5, strain
    limit 1%."""
    return Material(density=DENSITY, young_mod=E_PA / DENSITY, poiss_rat=0.25, bend=10.0,
                    strain_limit=0.01, contact_gap=1e-3, contact_offset=0.0, friction=0.5)


def _param(dt: float):
    p = default_param(dt)
    p.cg_tol = 1e-3
    return p


def cloth_sphere(side: int = 64, dt: float = 0.01):
    """One square sheet 1 m x 1 m as side x side vertices at y = 1.0,
    falling onto a fixed sphere of radius 0.3 at the origin."""
    v, f = meshes.grid(side, side, 1.0, 1.0)
    v[:, 1] = 1.0
    sc = Scene()
    sc.add_shell(v, f, cloth_material())
    sc.add_sphere((0.0, 0.0, 0.0), 0.3, contact_gap=1e-3, friction=0.5)
    return sc.build(_param(dt)), None


def _rot_y(v, angle):
    c, s = math.cos(angle), math.sin(angle)
    out = v.copy()
    out[:, 0] = c * v[:, 0] + s * v[:, 2]
    out[:, 2] = -s * v[:, 0] + c * v[:, 2]
    return out


def stacked_sheets(side: int = 128, sheets: int = 8, seed: int = 0, dt: float = 0.01,
                   cube: float = 0.6, gap: float = 0.02, collider: str = "mesh"):
    """`sheets` cloth sheets of side x side vertices (1 m), each rotated by a
    seeded uniform angle about the vertical, shifted by seeded uniform
    horizontal offsets in +-0.1 m, stacked `gap` apart above a fixed cube of
    side `cube` whose top face is at y = cube. The cube is a static collision
    mesh (`collider="mesh"`, the reference's representation) or a fully
    pinned shell (`collider="pinned"`)."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    mat = cloth_material()
    for k in range(sheets):
        v, f = meshes.grid(side, side, 1.0, 1.0)
        v = _rot_y(v.astype(np.float64), rng.uniform(0.0, 2.0 * math.pi))
        v[:, 0] += rng.uniform(-0.1, 0.1)
        v[:, 2] += rng.uniform(-0.1, 0.1)
        v[:, 1] = cube + gap * (k + 1)
        sc.add_shell(v.astype(np.float32), f, mat)
    cv, cf = meshes.box(cube, center=(0.0, 0.5 * cube, 0.0))
    if collider == "mesh":
        sc.add_collision_mesh(cv, cf, contact_gap=mat.contact_gap, friction=mat.friction)
    else:
        base = sc.add_shell(cv, cf, mat)
        sc.pin(np.arange(base, base + cv.shape[0]))
    return sc.build(_param(dt)), None


def twisted_tube(around: int = 256, along: int = 512, radius: float = 0.1,
                 length: float = 1.0, omega: float = 2.0, dt: float = 0.01):
    """Open tube along x; both end rings pinned as kinematic pins and rotated
    about the x axis in opposite directions at `omega` rad/s."""
    v, f = meshes.tube(around, along, radius, length)
    v[:, 1] += 0.5
    sc = Scene()
    sc.add_shell(v, f, cloth_material())
    left = np.arange(0, around)
    right = np.arange((along - 1) * around, along * around)
    pins = np.concatenate([left, right])
    sc.pin(pins, kinematic=True)
    rest = v[pins].astype(np.float64)
    sign = np.concatenate([np.full(around, 1.0), np.full(around, -1.0)])
    center_y, center_z = 0.5, 0.0

    def motion(t_end: float, step_dt: float):
        def at(t):
            ang = sign * omega * t
            c, s = np.cos(ang), np.sin(ang)
            y = rest[:, 1] - center_y
            z = rest[:, 2] - center_z
            out = rest.copy()
            out[:, 1] = center_y + c * y - s * z
            out[:, 2] = center_z + s * y + c * z
            return out

        p1 = at(t_end)
        p0 = at(t_end - step_dt)
        return p1.astype(np.float32), (p1 - p0).astype(np.float32)

    return sc.build(_param(dt)), motion


def sphere_field(side: int = 1024, spheres: int = 50, seed: int = 0, dt: float = 0.01,
                 height: float = 0.45):
    """A side x side sheet (1 m) at y = `height` over `spheres` fixed spheres
    with seeded radii U(0.02, 0.1) and centres uniform in the box
    [-0.5, 0.5] x [0, 0.3] x [-0.5, 0.5]."""
    rng = np.random.default_rng(seed)
    v, f = meshes.grid(side, side, 1.0, 1.0)
    v[:, 1] = height
    sc = Scene()
    sc.add_shell(v, f, cloth_material())
    for _ in range(spheres):
        c = (rng.uniform(-0.5, 0.5), rng.uniform(0.0, 0.3), rng.uniform(-0.5, 0.5))
        sc.add_sphere(c, rng.uniform(0.02, 0.1), contact_gap=1e-3, friction=0.5)
    return sc.build(_param(dt)), None


def cloth_drop(side: int, height: float, collider: str, size: float, dt: float = 0.01):
    """One 1 m square sheet of side x side vertices whose lowest point starts
    `height` above a fixed collider whose top is at y = 0: a sphere of radius
    `size` (the reference's analytic sphere) or a cube of side `size` (a static
    collision mesh). One scene of the batch of uneven drops."""
    v, f = meshes.grid(side, side, 1.0, 1.0)
    v[:, 1] = height
    sc = Scene()
    sc.add_shell(v, f, cloth_material())
    if collider == "sphere":
        sc.add_sphere((0.0, -size, 0.0), size, contact_gap=1e-3, friction=0.5)
    else:
        cv, cf = meshes.box(size, center=(0.0, -0.5 * size, 0.0))
        sc.add_collision_mesh(cv, cf, contact_gap=1e-3, friction=0.5)
    return sc.build(_param(dt)), None


def uneven_drops(count: int = 256, seed: int = 0):
    """The batch of uneven scenes: per scene a sheet side drawn log-uniformly
    from 16 to 96 vertices, a drop height uniform in [0.2, 1.0] m, and a
    collider drawn from a sphere of radius U(0.1, 0.4) m or a cube of side
    U(0.2, 0.6) m (seeded). Returns the parameters, not built scenes."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        side = int(round(math.exp(rng.uniform(math.log(16), math.log(96)))))
        height = float(rng.uniform(0.2, 1.0))
        if rng.random() < 0.5:
            out.append((side, height, "sphere", float(rng.uniform(0.1, 0.4))))
        else:
            out.append((side, height, "box", float(rng.uniform(0.2, 0.6))))
    return out


WORKLOADS = {
    "cloth_sphere": cloth_sphere,
    "stacked_sheets": stacked_sheets,
    "twisted_tube": twisted_tube,
    "sphere_field": sphere_field,
}
