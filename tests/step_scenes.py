"""Small seeded scenes for the step-level parity tests.

Each returns (scene, pin_motion) like ppf_gb300.scenes, sized so the CPU
oracle runs a step in well under a second.
"""
from __future__ import annotations

import math

import numpy as np

from ppf_gb300 import meshes, scenes
from ppf_gb300.session import Scene


def two_sheets(side: int = 12, gap: float = 6e-4, seed: int = 3, pinned: bool = True):
    """Two sheets inside each other's contact gap at t = 0, the upper one
    rotated and moving, the lower one pinned at two corners (unless not
    `pinned`), over a floor within reach: point-face, point-edge, point-point,
    edge-edge pairs, a floor constraint and Dirichlet rows in the first Newton
    system."""
    rng = np.random.default_rng(seed)
    mat = scenes.cloth_material()
    sc = Scene()
    va, fa = meshes.grid(side, side, 0.4, 0.4)
    va = va.astype(np.float64)
    va[:, 1] = 0.5 + rng.uniform(-5e-5, 5e-5, len(va))
    vb, fb = meshes.grid(side + 1, side - 1, 0.37, 0.41)
    vb = vb.astype(np.float64)
    c, s = math.cos(0.37), math.sin(0.37)
    x, z = vb[:, 0].copy(), vb[:, 2].copy()
    vb[:, 0] = c * x + s * z + 0.013
    vb[:, 2] = -s * x + c * z - 0.007
    vb[:, 1] = 0.5 + gap + rng.uniform(-5e-5, 5e-5, len(vb))
    a0 = sc.add_shell(va.astype(np.float32), fa, mat)
    b0 = sc.add_shell(vb.astype(np.float32), fb, mat)
    # a small triangle just below sheet A, one corner under A's far corner
    # (a point-point pair: neither projects into the other's interior)
    corner = va[side * side - 1]
    tri = np.array([[0.0, 0.0, 0.0], [0.05, 0.0, 0.01], [0.01, 0.0, 0.05]]) + corner
    tri[:, 1] = corner[1] - gap
    sc.add_shell(tri.astype(np.float32), np.array([[0, 2, 1]], np.uint32), mat)
    n = sc.vertex_count
    vel = np.zeros((n, 3), np.float32)
    vel[b0:b0 + len(vb)] = (0.2, -0.3, 0.1)
    sc.set_velocity(vel)
    if pinned:
        sc.pin([a0, a0 + side - 1])
    sc.add_floor((0.0, 0.5 - 8e-4, 0.0), contact_gap=1e-3, friction=0.5)
    return sc.build(scenes._param(0.01)), None


def cloth_on_box(side: int = 12, gap: float = 6e-4):
    """A sheet resting inside the contact gap of a static collision box's top
    face, rotated about the vertical and overhanging one top corner, so the
    first Newton system holds every collision-mesh contact: cloth vertices
    against the top face, the box corner against cloth faces and the box's top
    edges against cloth edges."""
    mat = scenes.cloth_material()
    sc = Scene()
    v, f = meshes.grid(side, side, 0.3, 0.3)
    v = v.astype(np.float64)
    c, s = math.cos(0.31), math.sin(0.31)
    x, z = v[:, 0].copy(), v[:, 2].copy()
    v[:, 0] = c * x + s * z + 0.04
    v[:, 2] = -s * x + c * z + 0.05
    v[:, 1] = 0.2 + gap
    sc.add_shell(v.astype(np.float32), f, mat)
    bv, bf = meshes.box(0.2, center=(0.0, 0.1, 0.0))
    sc.add_collision_mesh(bv, bf, contact_gap=1e-3, friction=0.5)
    return sc.build(scenes._param(0.01)), None


def sheet_on_sphere(side: int = 20):
    """cloth_sphere at a reduced size, lowered to just above the sphere."""
    sc, mot = scenes.cloth_sphere(side)
    return sc, mot


def strain_of(x, rest, faces):
    """Largest singular value of each face's deformation gradient relative to
    its rest triangle (the quantity the 1% strain limit bounds)."""
    x = np.asarray(x, np.float64)
    rest = np.asarray(rest, np.float64)
    f = np.asarray(faces, np.int64)
    r1 = rest[f[:, 1]] - rest[f[:, 0]]
    r2 = rest[f[:, 2]] - rest[f[:, 0]]
    e1 = r1 / np.linalg.norm(r1, axis=1, keepdims=True)
    nrm = np.cross(r1, r2)
    e2 = np.cross(nrm, r1)
    e2 /= np.linalg.norm(e2, axis=1, keepdims=True)
    Dm = np.stack([np.stack([(e1 * r1).sum(1), (e2 * r1).sum(1)], 1),
                   np.stack([(e1 * r2).sum(1), (e2 * r2).sum(1)], 1)], 2)  # [F,2,2] cols
    Ds = np.stack([x[f[:, 1]] - x[f[:, 0]], x[f[:, 2]] - x[f[:, 0]]], 2)  # [F,3,2]
    F = Ds @ np.linalg.inv(Dm)
    return np.linalg.svd(F, compute_uv=False)[:, 0]


def rod_material(**kw):
    from ppf_gb300.session import RodMaterial

    base = dict(density=0.01, young_mod=1e4, bend=0.5, contact_gap=1e-3, friction=0.3,
                strain_limit=0.01)
    base.update(kw)
    return RodMaterial(**base)


def rods_and_sheet(seed: int = 4):
    """Three rods and a sheet, every rod term active in the first Newton
    system: rod A lies across the sheet inside its contact gap, stretched
    0.4 % (the rod strain limit is 1 %) and damped; rod B is a zigzag that
    keeps its bent rest shape, crossing rod A within the gap and falling;
    rod C hangs off the sheet's edge with bending damping. The sheet has
    membrane and bending damping. No pins: the system before and after the
    Dirichlet elimination is the same."""
    rng = np.random.default_rng(seed)
    mat = scenes.cloth_material()
    mat.deform_damping = 0.05
    mat.bend_damping = 0.02
    sc = Scene()
    v, f = meshes.grid(10, 10, 0.2, 0.2)
    v = v.astype(np.float64)
    v[:, 1] = 0.5 + rng.uniform(-2e-5, 2e-5, len(v))
    sc.add_shell(v.astype(np.float32), f, mat)
    # rod A: along x across the sheet, 6e-4 above it
    na = 24
    xa = np.stack([np.linspace(-0.12, 0.12, na), np.full(na, 0.5 + 6e-4),
                   np.linspace(-0.01, 0.013, na)], 1)
    ea = np.stack([np.arange(na - 1), np.arange(1, na)], 1)
    a0 = sc.add_rod(xa.astype(np.float32), ea, rod_material(deform_damping=0.1))
    # rod B: zigzag along z, crossing rod A 7e-4 above it
    nb = 16
    zb = np.linspace(-0.08, 0.08, nb)
    xb = np.stack([0.01 + 0.006 * (np.arange(nb) % 2), np.full(nb, 0.5 + 13e-4), zb], 1)
    eb = np.stack([np.arange(nb - 1), np.arange(1, nb)], 1)
    b0 = sc.add_rod(xb.astype(np.float32), eb,
                    rod_material(bend=2.0, bend_rest_from_geometry=True, bend_damping=0.05))
    # rod C: off the sheet's edge, bent downward
    nc = 12
    t = np.linspace(0.0, 1.0, nc)
    xc = np.stack([0.105 + 0.05 * t, 0.5 - 0.03 * t * t, np.full(nc, 0.02)], 1)
    ec = np.stack([np.arange(nc - 1), np.arange(1, nc)], 1)
    sc.add_rod(xc.astype(np.float32), ec, rod_material(bend=1.0, bend_damping=0.1))
    n = sc.vertex_count
    vel = np.zeros((n, 3), np.float32)
    vel[b0:b0 + nb] = (0.0, -0.2, 0.05)
    vel[:a0] = (0.0, -0.05, 0.0)
    sc.set_velocity(vel)
    sc.add_floor((0.0, 0.3, 0.0), contact_gap=1e-3, friction=0.5)
    built = sc.build(scenes._param(0.01))
    # stretch rod A by 0.4 % about its centre (its strain barrier is active)
    curr, prev = built.positions()
    c = curr[a0:a0 + na].mean(axis=0)
    curr[a0:a0 + na] = c + 1.004 * (curr[a0:a0 + na] - c)
    prev[a0:a0 + na] = c + 1.004 * (prev[a0:a0 + na] - c)
    built.set_positions(curr, prev)
    return built, {"rod_a": (a0, na), "rod_b": (b0, nb)}


def solids_and_sheet(seed: int = 6):
    """Two solids and a sheet, every solid term active in the first Newton
    system: an ARAP block (3^3 cells, eight interior vertices, sheared and
    damped) with a sheet lying 6e-4 above its top face, and a falling SNHk
    block (2^3 cells) whose corner is within the gap of the first's side; an
    StVK sheet membrane exercises the shell models. No pins."""
    from ppf_gb300.session import SolidMaterial

    rng = np.random.default_rng(seed)
    sc = Scene()
    va, ta = meshes.tet_box(3, 0.1, center=(0.0, 0.45, 0.0))
    a0 = sc.add_solid(va, ta, SolidMaterial(model=0, density=500.0, young_mod=800.0,
                                            poiss_rat=0.3, contact_gap=1e-3, friction=0.4,
                                            deform_damping=0.05))
    vb, tb = meshes.tet_box(2, 0.05, center=(0.0778, 0.47, 0.03))
    vb = vb + rng.uniform(-2e-4, 2e-4, vb.shape).astype(np.float32)
    b0 = sc.add_solid(vb, tb, SolidMaterial(model=3, density=800.0, young_mod=600.0,
                                            poiss_rat=0.35, contact_gap=1e-3, friction=0.2))
    mat = scenes.cloth_material()
    mat.model = 1  # StVK
    vs, fs = meshes.grid(8, 8, 0.12, 0.12)
    vs = vs.astype(np.float64)
    vs[:, 1] = 0.5 + 6e-4 + rng.uniform(-2e-5, 2e-5, len(vs))
    sc.add_shell(vs.astype(np.float32), fs, mat)
    n = sc.vertex_count
    vel = np.zeros((n, 3), np.float32)
    vel[b0:b0 + len(vb)] = (0.0, -0.3, 0.0)
    sc.set_velocity(vel)
    sc.add_floor((0.0, 0.3, 0.0), contact_gap=1e-3, friction=0.5)
    built = sc.build(scenes._param(0.01))
    # shear block A by 3 % (curr and prev alike: its elastic force is active)
    curr, prev = built.positions()
    for arr in (curr, prev):
        blk = arr[a0:a0 + len(va)]
        blk[:, 0] += 0.03 * (blk[:, 1] - 0.45)
    built.set_positions(curr, prev)
    return built, {"block_a": (a0, len(va)), "block_b": (b0, len(vb))}


def stitched_sheets(seed: int = 8):
    """Two sheets side by side, 2 mm apart, stitched along their facing
    edges: each of sheet A's edge vertices to the barycentric point of the
    nearest face of sheet B (vertex-to-face stitches), and B's corner
    vertices to A's (vertex-to-vertex), with two stiffnesses. No pins."""
    rng = np.random.default_rng(seed)
    mat = scenes.cloth_material()
    sc = Scene()
    side = 8
    va, fa = meshes.grid(side, side, 0.1, 0.1)
    va = va.astype(np.float64)
    va[:, 0] -= 0.051
    va[:, 1] = 0.5 + rng.uniform(-1e-5, 1e-5, len(va))
    vb = va.copy()
    vb[:, 0] += 0.102
    a0 = sc.add_shell(va.astype(np.float32), fa, mat)
    b0 = sc.add_shell(vb.astype(np.float32), fa, mat)
    # A's right edge (x max) to B's left-edge faces
    right = [j * side + side - 1 for j in range(side)]
    left_faces = [k for k, f in enumerate(fa) if min(vb[f][:, 0]) < vb[:, 0].min() + 1e-9]
    for v in right:
        f = fa[left_faces[min(range(len(left_faces)),
                               key=lambda k: np.linalg.norm(vb[fa[left_faces[k]]].mean(0) - va[v]))]]
        w = rng.dirichlet([4.0, 4.0, 4.0]).astype(np.float32)
        sc.add_stitch([a0 + v] * 3 + [b0 + int(t) for t in f], [1.0, 0.0, 0.0, *w], 0.8)
    for v in (0, (side - 1) * side):
        sc.add_stitch([b0 + v] * 3 + [a0 + v + side - 1] * 3, [1.0, 0.0, 0.0, 1.0, 0.0, 0.0],
                      1.5)
    n = sc.vertex_count
    vel = np.zeros((n, 3), np.float32)
    vel[b0:] = (0.05, -0.02, 0.0)
    sc.set_velocity(vel)
    return sc.build(scenes._param(0.01)), None
