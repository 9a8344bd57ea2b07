"""The C++ scene builder against a numpy restatement of the reference's Rust
builder (CPU only).

The builder (csrc/host/builder.cpp) produces the DataSet that both the
library and every oracle consume, so an error there would be invisible to
the parity tests. Here each of its arrays is recomputed in numpy, from the
Rust source, with float32 arithmetic rounded at every operation as the Rust
code's f32 (nalgebra) arithmetic is:

* face area 0.5 |(x1 - x0) x (x2 - x0)| and mass density * area
  (triutils.rs:9-17, scene.rs:1661, 1798);
* Lame parameters from (E, nu) (builder.rs:1739-1743);
* lumped vertex area and mass, a third of each face's, added face by face
  and corner by corner (builder.rs:571-606);
* inverse rest matrices in the face's tangent frame: e1 = d0 / |d0|,
  e2 = normalize(n x d0), the 2 x 2 matrix of projections and its inverse
  by the cofactor formula (builder.rs:157-230, nalgebra's normalize divides
  and its 2 x 2 try_inverse is m22 / det, -m12 / det, -m21 / det, m11 / det);
* edges keyed by their vertex pair, oriented as in their first face, with
  their first two faces (mesh.rs:188-229), and hinges (shared edge as in the
  first face, its opposite corner, the second face's opposite corner; edges
  of more than two faces carry none; mesh.rs:231-293). The reference emits
  both in hash-map order, the builder in first-seen order, so they are
  compared as keyed sets;
* the upper-triangle fixed pattern with each row sorted, its transpose table
  and the face / hinge slot tables, hinges in the (2, 1, 0, 3) remapped order
  (builder.rs:1244-1420);
* hinge length |x(h0) - x(h1)| and area (the two faces' areas summed)
  (builder.rs:872-905).

Integer arrays are compared exactly and float arrays bit for bit.
"""
import math

import numpy as np
import pytest

import step_scenes
from ppf_gb300 import meshes, scenes

f32 = np.float32


def _cross(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1)


def _dot(a, b):
    return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]


def _norm(a):
    return np.sqrt(_dot(a, a))


def restate(x, faces, density, young, poisson):
    """The reference builder's arrays for one shell material."""
    x = np.asarray(x, f32)
    F = np.asarray(faces, np.int64)
    n, nf = len(x), len(F)
    out = {}
    e0 = x[F[:, 1]] - x[F[:, 0]]
    e1 = x[F[:, 2]] - x[F[:, 0]]
    area = f32(0.5) * _norm(_cross(e0, e1))
    out["face_area"] = area
    out["face_mass"] = f32(density) * area
    E, nu = f32(young), f32(poisson)
    out["face_mu"] = np.full(nf, E / (f32(2.0) * (f32(1.0) + nu)), f32)
    out["face_lambda"] = np.full(nf, E * nu / ((f32(1.0) + nu) * (f32(1.0) - f32(2.0) * nu)),
                                 f32)
    va = np.zeros(n, f32)
    vm = np.zeros(n, f32)
    third_a = area / f32(3.0)
    third_m = out["face_mass"] / f32(3.0)
    for i in range(nf):  # face by face, corner by corner
        for k in range(3):
            va[F[i, k]] += third_a[i]
    for i in range(nf):
        for k in range(3):
            vm[F[i, k]] += third_m[i]
    out["vertex_area"], out["vertex_mass"] = va, vm
    # inverse rest matrices
    d0, d1 = e0, e1
    nn = _cross(d0, d1)
    e2 = _cross(nn, d0)
    e2 = e2 / _norm(e2)[:, None]
    u1 = d0 / _norm(d0)[:, None]
    a, b = _dot(u1, d0), _dot(u1, d1)
    c, d = _dot(e2, d0), _dot(e2, d1)
    det = a * d - c * b
    out["inv_rest2x2"] = np.stack([d / det, -c / det, -b / det, a / det], 1).reshape(-1)
    # edges and hinges
    edges, hinges = {}, {}
    for i in range(nf):
        f = F[i]
        for j in range(3):
            p, q, o = int(f[j]), int(f[(j + 1) % 3]), int(f[(j + 2) % 3])
            key = (min(p, q), max(p, q))
            if key in edges:
                if len(edges[key][1]) < 2:
                    edges[key][1].append(i)
            else:
                edges[key] = ((p, q), [i])
            h = hinges.get(key)
            if h is None:
                hinges[key] = [p, q, o, None, i, None, 1]
            else:
                if h[6] == 1:
                    h[3], h[5] = o, i
                h[6] += 1
    out["edges"] = {k: (v[0], tuple(v[1])) for k, v in edges.items()}
    out["hinges"] = {k: (tuple(h[:4]), (h[4], h[5])) for k, h in hinges.items() if h[6] == 2}
    # fixed pattern, transpose, slots
    rows = [set([i]) for i in range(n)]

    def ins(i, j):
        if i <= j:
            rows[i].add(j)

    for (p, q), _ in out["edges"].values():
        for s in (p, q):
            for t in (p, q):
                ins(s, t)
    for f in F:
        for s in f:
            for t in f:
                ins(int(s), int(t))
    for h, _ in out["hinges"].values():
        for s in h:
            for t in h:
                ins(s, t)
    rows = [sorted(r) for r in rows]
    off = np.zeros(n + 1, np.uint32)
    off[1:] = np.cumsum([len(r) for r in rows])
    out["fixed_offset"] = off
    out["fixed_index"] = np.array([j for r in rows for j in r], np.uint32)
    tr = [[] for _ in range(n)]
    for i, r in enumerate(rows):
        for k, j in enumerate(r):
            if j != i:
                tr[j].append((i, int(off[i]) + k))
    out["transpose"] = np.array([v for t in tr for p in t for v in p], np.uint32)
    pos = [{j: int(off[i]) + k for k, j in enumerate(r)} for i, r in enumerate(rows)]

    def slot(i, j):
        return 0xFFFFFFFF if i > j else pos[i][j]

    out["face_slots"] = np.array([slot(int(s), int(t)) for f in F for s in f for t in f],
                                 np.uint32)
    out["hinge_slots"] = {}
    out["hinge_length"], out["hinge_area"] = {}, {}
    for key, (h, fs) in out["hinges"].items():
        r = (h[2], h[1], h[0], h[3])
        out["hinge_slots"][key] = tuple(slot(s, t) for s in r for t in r)
        dv = (x[h[0]] - x[h[1]])[None]
        out["hinge_length"][key] = _norm(dv)[0]
        out["hinge_area"][key] = f32(f32(0.0) + area[fs[0]]) + area[fs[1]]
    return out


def _check(sc, x, faces, mat):
    ref = restate(x, faces, mat.density, mat.young_mod, mat.poiss_rat)
    for name in ("face_area", "face_mass", "face_mu", "face_lambda", "vertex_area",
                 "vertex_mass", "inv_rest2x2"):
        got = sc.array(name)
        assert got.dtype == np.float32
        bad = np.flatnonzero(got.view(np.uint32) != ref[name].astype(f32).view(np.uint32))
        assert bad.size == 0, (name, bad[:5], got[bad[:5]], ref[name][bad[:5]])
    for name in ("fixed_offset", "fixed_index", "transpose", "face_slots"):
        assert np.array_equal(sc.array(name), ref[name]), name
    # edges: oriented pair and incident faces per key
    E = sc.array("edge").reshape(-1, 2)
    eoff, ef = sc.array("edge_face_offset"), sc.array("edge_face")
    got_e = {}
    for i, (p, q) in enumerate(E.tolist()):
        got_e[(min(p, q), max(p, q))] = ((p, q), tuple(ef[eoff[i]:eoff[i + 1]].tolist()))
    assert got_e == ref["edges"]
    # hinges: vertex tuple, slots, length and area per key
    H = sc.array("hinge").reshape(-1, 4)
    hs = sc.array("hinge_slots").reshape(-1, 16)
    hl, ha = sc.array("hinge_length"), sc.array("hinge_area")
    assert len(H) == len(ref["hinges"])
    for i, h in enumerate(H.tolist()):
        key = (min(h[0], h[1]), max(h[0], h[1]))
        assert tuple(h) == ref["hinges"][key][0], key
        assert tuple(hs[i].tolist()) == ref["hinge_slots"][key], key
        assert hl[i].view(np.uint32) == ref["hinge_length"][key].view(np.uint32), key
        assert ha[i].view(np.uint32) == f32(ref["hinge_area"][key]).view(np.uint32), key


def test_builder_matches_restated_reference_on_a_sheet(product_lib):
    v, f = meshes.grid(17, 13, 0.7, 0.5)
    v = v.astype(np.float64)
    rng = np.random.default_rng(5)
    v += rng.uniform(-0.004, 0.004, v.shape)  # irregular triangles
    v = v.astype(np.float32)
    mat = scenes.cloth_material()
    from ppf_gb300.session import Scene

    sc = Scene()
    sc.add_shell(v, f, mat)
    sc.build(scenes._param(0.01))
    _check(sc, v, f, mat)


def test_builder_matches_restated_reference_on_stacked_sheets(product_lib):
    sc, _ = scenes.stacked_sheets(side=20, sheets=3, seed=2)
    x = sc.positions()[0]
    faces = sc.array("face").reshape(-1, 3)
    _check(sc, x, faces, scenes.cloth_material())


def test_builder_matches_restated_reference_with_pins(product_lib):
    """The two-sheet scene (three shells, pinned corners): pins change only
    the fixed flags, which the element tests cover; the arrays here must
    still be the reference builder's."""
    sc, _ = step_scenes.two_sheets()
    x = sc.positions()[0]
    faces = sc.array("face").reshape(-1, 3)
    _check(sc, x, faces, scenes.cloth_material())


def test_non_manifold_edge_carries_no_hinge(product_lib):
    """Three triangles on one edge: the edge keeps its first two faces and
    no hinge is made for it (mesh.rs:206-212, 271-279)."""
    from ppf_gb300.session import Scene

    v = np.array([[0, 0, 0], [1, 0, 0], [0.5, 1, 0], [0.5, -1, 0], [0.5, 0, 1]], np.float32)
    f = np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4]], np.uint32)
    mat = scenes.cloth_material()
    sc = Scene()
    sc.add_shell(v, f, mat)
    sc.build(scenes._param(0.01))
    _check(sc, v, f, mat)
    H = sc.array("hinge").reshape(-1, 4)
    assert not any({0, 1} <= set(h[:2]) for h in H.tolist())
