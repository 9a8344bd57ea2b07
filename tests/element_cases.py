"""Seeded element-level cases: inputs, calling convention and tolerances.

Shared by tests/golden/make_golden.py (which evaluates the reference's own
element code, compiled from its sources into oracle/_ref/libppfref.so, and
freezes the outputs) and by tests/test_elements.py (which evaluates the same
inputs through the element math the CUDA kernels use, compiled for the CPU in
oracle/liboracle_ppf.so, and compares).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

f32 = np.float32


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _sym(rng, n, scale=1.0):
    a = rng.normal(0, scale, (n, n))
    return (a + a.T).astype(f32)


def _spd(rng, n, scale=1.0):
    a = rng.normal(0, scale, (n, n))
    return (a @ a.T + 0.1 * np.eye(n)).astype(f32)


def _F(rng, s=0.05):
    return (np.eye(3, 2) + rng.normal(0, s, (3, 2))).astype(f32)


def _colmajor(m):
    return np.ascontiguousarray(np.asarray(m, f32).T).reshape(-1)


# Each case generator returns a dict of named float32 input arrays / scalars.
def gen_distance(rng, n):
    out = []
    for _ in range(n):
        p = rng.normal(0, 1, (5, 3)).astype(f32)
        out.append({"p": p[0], "a": p[1], "b": p[2], "c": p[3], "d": p[4]})
    return out


def gen_barrier(rng, n):
    out = []
    for _ in range(n):
        ghat = f32(10 ** rng.uniform(-4, -2))
        off = f32(rng.choice([0.0, 1e-4]))
        g = f32(off + rng.uniform(0.05, 1.5) * ghat)
        e = rng.normal(0, 1, 3)
        e = (e / np.linalg.norm(e) * g).astype(f32)
        out.append({"g": g, "ghat": ghat, "off": off, "e": e, "kind": 0})
    return out


def gen_stiffness(rng, n):
    out = []
    for i in range(n):
        k = 2 + i % 3
        w = rng.normal(0, 1, k).astype(f32)
        w[0] = 1.0
        w[1:] = -np.abs(w[1:]) / np.abs(w[1:]).sum()
        mass = rng.uniform(1e-4, 1e-3, k).astype(f32)
        if i % 5 == 0:
            mass[-1] = 0.0
        e = rng.normal(0, 1e-3, 3).astype(f32)
        out.append({"n": k, "w": w, "mass": mass, "local": _colmajor(_spd(rng, 3 * k, 10.0)),
                    "e": e, "ghat": f32(1e-3), "off": f32(0.0)})
    return out


def gen_friction(rng, n):
    out = []
    for i in range(n):
        nrm = rng.normal(0, 1, 3)
        nrm = (nrm / np.linalg.norm(nrm)).astype(f32)
        force = (-nrm * rng.uniform(0.1, 10)).astype(f32)
        scale = 1e-6 if i % 2 else 1e-3
        out.append({"force": force, "dx": rng.normal(0, scale, 3).astype(f32),
                    "normal": nrm, "mu": f32(0.5), "eps": f32(1e-5)})
    return out


def gen_F(rng, n):
    out = []
    for i in range(n):
        F = _F(rng, 0.02 if i % 2 else 0.2)
        if i % 7 == 0:  # axis-aligned column: exercises the candidate ties
            F[:, 0] = [0.0, 0.0, 1.0 + 0.01 * i / n]
        out.append({"F": _colmajor(F), "mu": f32(rng.uniform(10, 1e4)),
                    "lmd": f32(rng.uniform(10, 1e4))})
    return out


def gen_convert(rng, n):
    out = []
    for _ in range(n):
        x = rng.normal(0, 0.01, (3, 3)).astype(f32)
        inv = (rng.normal(0, 1, (2, 2)) + 60 * np.eye(2)).astype(f32)
        out.append({"x0": x[0], "x1": x[1], "x2": x[2], "inv": _colmajor(inv),
                    "dedF": rng.normal(0, 1, 6).astype(f32),
                    "d2": _colmajor(_sym(rng, 6))})
    return out


def gen_hinge(rng, n):
    out = []
    for i in range(n):
        # shared edge h0-h1 along x, flaps h2 / h3 on either side, bent by an
        # angle that ranges from nearly flat to strongly folded
        ang = rng.uniform(-2.5, 2.5) if i % 3 else rng.uniform(-0.05, 0.05)
        h0 = np.array([0.0, 0.0, 0.0])
        h1 = np.array([1.0, 0.0, 0.0])
        h2 = np.array([rng.uniform(0.2, 0.8), 0.0, rng.uniform(0.5, 1.0)])
        r = rng.uniform(0.5, 1.0)
        h3 = np.array([rng.uniform(0.2, 0.8), r * np.sin(ang), -r * np.cos(ang)])
        x = (np.stack([h0, h1, h2, h3]) * 0.01 + rng.normal(0, 1e-4, (4, 3))).astype(f32)
        out.append({"x": x.reshape(-1), "rest": f32(rng.uniform(-0.3, 0.3) if i % 4 == 0 else 0.0)})
    return out


def gen_rod(rng, n):
    """Rod edges stretched and compressed against their rest length, and rod
    vertices bent from straight (including exactly and nearly collinear
    triples) to folded, with straight and bent rest angles."""
    out = []
    for i in range(n):
        x0 = rng.normal(0, 0.01, 3)
        d = rng.normal(0, 1, 3)
        d /= np.linalg.norm(d)
        l0 = rng.uniform(0.005, 0.02)
        x1 = x0 + d * l0 * rng.uniform(0.7, 1.3)
        ang = [np.pi, np.pi - 1e-4, rng.uniform(0.3, np.pi)][i % 3]
        a = rng.normal(0, 1, 3)
        a /= np.linalg.norm(a)
        b = np.cross(a, rng.normal(0, 1, 3))
        b /= np.linalg.norm(b)
        la, lb = rng.uniform(0.005, 0.02, 2)
        c = rng.normal(0, 0.01, 3)
        p0 = c + la * a
        p2 = c + lb * (np.cos(ang) * a + np.sin(ang) * b)
        rest = [np.pi, rng.uniform(1.0, np.pi), rng.uniform(0.5, 2.5)][i % 3]
        out.append({"x0": x0.astype(f32), "x1": x1.astype(f32), "l0": f32(l0),
                    "w": f32(10 ** rng.uniform(-2, 3)),
                    "b": np.stack([p0, c, p2]).astype(f32), "rest": f32(rest)})
    return out


def gen_solid(rng, n):
    """Tets and shell faces deformed around their rest shape (some inverted,
    so the rotation-variant SVD flips a sign), under ARAP, StVK and SNHk."""
    out = []
    for i in range(n):
        rest = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64) * 0.02
        rest += rng.normal(0, 0.003, rest.shape)
        D = (rest[1:] - rest[0]).T
        inv = np.linalg.inv(D)
        A = np.eye(3) + rng.normal(0, 0.15, (3, 3))
        if i % 5 == 0:
            A[:, 2] *= -0.3  # inverted
        x = rest[0] + (A @ (rest - rest[0]).T).T + rng.normal(0, 0.01, 3)
        F = (A + rng.normal(0, 0.05, (3, 3))).astype(f32)
        tri = x[:3].copy()
        d2 = np.stack([tri[1] - tri[0], tri[2] - tri[0]], 1)
        inv2 = np.linalg.inv(np.array([[np.linalg.norm(d2[:, 0]), 0.0],
                                       [0.0, np.linalg.norm(d2[:, 1])]]) + rng.normal(0, 0.01, (2, 2)))
        out.append({"model": [0, 1, 3][i % 3], "mu": f32(10 ** rng.uniform(2, 4)),
                    "lmd": f32(10 ** rng.uniform(2, 4)), "mass": f32(rng.uniform(0.01, 1.0)),
                    "x": x.astype(f32).reshape(-1), "inv": inv.T.astype(f32).reshape(-1),
                    "F": F.T.reshape(-1).copy(), "a3": (1.0 + rng.normal(0, 0.2, 3)).astype(f32),
                    "tri": tri.astype(f32).reshape(-1), "inv2": inv2.T.astype(f32).reshape(-1)})
    return out


def gen_sym(rng, n):
    out = []
    for i in range(n):
        a3 = _sym(rng, 3, 10 ** rng.uniform(-3, 3))
        if i % 6 == 0:
            a3 = (np.eye(3) * 5.0 + 1e-7 * rng.normal(0, 1, (3, 3))).astype(f32)
            a3 = (a3 + a3.T) / 2
        out.append({"A2": _colmajor(_sym(rng, 2)), "A3": _colmajor(a3),
                    "A4": _colmajor(_sym(rng, 4)), "spd3": _colmajor(_spd(rng, 3))})
    return out


def gen_strain(rng, n):
    out = []
    for i in range(n):
        F = _F(rng, 0.01)
        F[:, 0] *= 1.0 + rng.uniform(0.0, 0.012)
        U, S, Vt = np.linalg.svd(F.astype(np.float64), full_matrices=False)
        S = S[::-1].copy()
        U = U[:, ::-1].copy()
        Vt = Vt[::-1, :].copy()
        a = (S - 1.0).astype(f32)
        out.append({"F": _colmajor(F), "a": a, "ghat": f32(0.01),
                    "U": _colmajor(U), "S": S.astype(f32), "Vt": _colmajor(Vt),
                    "eps": f32(1e-2), "x": rng.normal(0, 0.01, 9).astype(f32),
                    "local": _colmajor(_spd(rng, 9, 10.0)), "mass": f32(1e-4),
                    "limit": f32(0.01)})
    return out


def gen_ccd(rng, n):
    out = []
    for i in range(n):
        kind = i % 4
        tri = rng.normal(0, 0.05, (3, 3))
        tri[:, 1] = rng.normal(0, 1e-3, 3)
        p0 = np.array([rng.uniform(-0.01, 0.01), rng.uniform(2e-3, 3e-2), rng.uniform(-0.01, 0.01)])
        move = np.array([rng.normal(0, 0.01), -rng.uniform(0.0, 0.06), rng.normal(0, 0.01)])
        cols0 = np.vstack([p0, tri])
        cols1 = cols0.copy()
        cols1[0] += move
        cols1[1:] += rng.normal(0, 1e-3, (3, 3))
        if kind == 3:  # edge-edge: crossing edges, one above the other
            cols0 = np.array([[-0.05, p0[1], 0.0], [0.05, p0[1], 0.0],
                              [0.0, 0.0, -0.05], [0.0, 0.0, 0.05]]) + rng.normal(0, 1e-3, (4, 3))
            cols1 = cols0.copy()
            cols1[:2] += move
        out.append({"kind": kind, "x0": cols0.astype(f32).reshape(-1),
                    "x1": cols1.astype(f32).reshape(-1),
                    "off": f32(0.0 if i % 3 else 1e-4), "ghat": f32(1e-3),
                    "max_t": f32(1.25), "eps": f32(1e-7)})
    return out


def gen_isect(rng, n):
    out = []
    for _ in range(n):
        t = rng.normal(0, 1, (3, 3)).astype(f32)
        e = rng.normal(0, 1, (2, 3)).astype(f32)
        out.append({"t": t, "e": e})
    return out


# ---------------------------------------------------------------------------
# Evaluation: `lib` is the ref (prefix "ref_") or oracle (prefix "orc_").
def evaluate(lib, prefix, rng_seed=7, n=64):
    rng = np.random.default_rng(rng_seed)
    fn = lambda name: getattr(lib, prefix + name)  # noqa: E731
    res = {}

    def rec(name, i, **outs):
        for k, v in outs.items():
            res.setdefault(f"{name}.{k}", []).append(np.asarray(v, f32).reshape(-1))

    for i, c in enumerate(gen_distance(rng, n)):
        for name, args, m in (("pe_coeff", ("p", "a", "b"), 2),
                              ("pt_coeff", ("p", "a", "b", "c"), 3),
                              ("ee_coeff", ("p", "a", "b", "c"), 4),
                              ("pt_coeff_unclassified", ("p", "a", "b", "c"), 3),
                              ("pe_coeff_unclassified", ("p", "a", "b"), 2)):
            o = np.zeros(m, f32)
            fn(name)(*[_ptr(c[a]) for a in args], _ptr(o))
            rec(name, i, out=o)
    for i, c in enumerate(gen_barrier(rng, n)):
        o = np.zeros(3, f32)
        f = fn("barrier")
        f.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float)]
        f(0, c["g"], c["ghat"], c["off"], _ptr(o))
        g = np.zeros(3, f32)
        h = np.zeros(9, f32)
        f2 = fn("edge_grad_hess")
        f2.argtypes = [C.POINTER(C.c_float), C.c_float, C.c_float, C.c_int,
                       C.POINTER(C.c_float), C.POINTER(C.c_float)]
        f2(_ptr(c["e"]), c["ghat"], c["off"], 0, _ptr(g), _ptr(h))
        rec("barrier", i, val=o, edge_g=g, edge_h=h)
    for i, c in enumerate(gen_stiffness(rng, n)):
        f = fn("stiffness")
        f.restype = C.c_float
        f.argtypes = [C.c_int] + [C.POINTER(C.c_float)] * 4 + [C.c_float, C.c_float]
        v = f(c["n"], _ptr(c["w"]), _ptr(c["mass"]), _ptr(c["local"]), _ptr(c["e"]),
              c["ghat"], c["off"])
        rec("stiffness", i, k=[v])
    for i, c in enumerate(gen_friction(rng, n)):
        g = np.zeros(3, f32)
        h = np.zeros(9, f32)
        f = fn("friction")
        f.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_float, C.c_float] + [C.POINTER(C.c_float)] * 2
        f(_ptr(c["force"]), _ptr(c["dx"]), _ptr(c["normal"]), c["mu"], c["eps"], _ptr(g), _ptr(h))
        pg = np.zeros(3, f32)
        ph = np.zeros(9, f32)
        e = (-c["normal"] * f32(5e-4)).astype(f32)
        fp = fn("push")
        fp.argtypes = [C.POINTER(C.c_float)] * 2 + [C.c_float] + [C.POINTER(C.c_float)] * 2
        fp(_ptr(e), _ptr(c["normal"]), f32(1e-3), _ptr(pg), _ptr(ph))
        rec("friction", i, g=g, h=h, push_g=pg, push_h=ph)
    for i, c in enumerate(gen_F(rng, n)):
        sg, sh, hg, hh = (np.zeros(k, f32) for k in (6, 36, 6, 36))
        f = fn("bw")
        f.argtypes = [C.POINTER(C.c_float), C.c_float, C.c_float] + [C.POINTER(C.c_float)] * 4
        f(_ptr(c["F"]), c["mu"], c["lmd"], _ptr(sg), _ptr(sh), _ptr(hg), _ptr(hh))
        rec("bw", i, stretch_g=sg, stretch_h=sh, shear_g=hg, shear_h=hh)
    for i, c in enumerate(gen_convert(rng, n)):
        F6 = np.zeros(6, f32)
        fn("deformation_grad")(_ptr(c["x0"]), _ptr(c["x1"]), _ptr(c["x2"]), _ptr(c["inv"]), _ptr(F6))
        f9 = np.zeros(9, f32)
        h81 = np.zeros(81, f32)
        fn("convert")(_ptr(c["dedF"]), _ptr(c["d2"]), _ptr(c["inv"]), _ptr(f9), _ptr(h81))
        rec("convert", i, F=F6, f=f9, h=h81)
    for i, c in enumerate(gen_hinge(rng, n)):
        ang = np.zeros(1, f32)
        f12 = np.zeros(12, f32)
        h144 = np.zeros(144, f32)
        f = fn("hinge")
        f.argtypes = [C.POINTER(C.c_float), C.c_float] + [C.POINTER(C.c_float)] * 3
        f(_ptr(c["x"]), c["rest"], _ptr(ang), _ptr(f12), _ptr(h144))
        rec("hinge", i, angle=ang, f=f12, h=h144)
    for i, c in enumerate(gen_sym(rng, n)):
        v2, e2 = np.zeros(2, f32), np.zeros(4, f32)
        fn("symm2")(_ptr(c["A2"]), _ptr(v2), _ptr(e2))
        v3, e3 = np.zeros(3, f32), np.zeros(9, f32)
        fn("symm3")(_ptr(c["A3"]), _ptr(v3), _ptr(e3))
        a4 = c["A4"].copy()
        fn("psd4")(_ptr(a4))
        rec("eig", i, val2=v2, vec2=e2, val3=v3, vec3=e3, psd4=a4)
    for i, c in enumerate(gen_strain(rng, n)):
        U6, S2, Vt4 = np.zeros(6, f32), np.zeros(2, f32), np.zeros(4, f32)
        fn("svd32")(_ptr(c["F"]), _ptr(U6), _ptr(S2), _ptr(Vt4))
        deda, d2 = np.zeros(2, f32), np.zeros(4, f32)
        f = fn("strainlimit_table")
        f.argtypes = [C.POINTER(C.c_float), C.c_float, C.c_int] + [C.POINTER(C.c_float)] * 2
        f(_ptr(c["a"]), c["ghat"], 0, _ptr(deda), _ptr(d2))
        f6, h36 = np.zeros(6, f32), np.zeros(36, f32)
        f = fn("eigen_force_hessian")
        f.argtypes = [C.POINTER(C.c_float)] * 5 + [C.c_float] + [C.POINTER(C.c_float)] * 2
        f(_ptr(deda), _ptr(d2), _ptr(c["U"]), _ptr(c["S"]), _ptr(c["Vt"]), c["eps"], _ptr(f6), _ptr(h36))
        fs = fn("strain_stiffness")
        fs.restype = C.c_float
        fs.argtypes = [C.POINTER(C.c_float)] * 2 + [C.c_float, C.POINTER(C.c_float), C.c_float]
        k = fs(_ptr(c["x"]), _ptr(c["local"]), c["mass"], _ptr(c["a"]), c["limit"])
        fm = fn("singular_minus_one_max")
        fm.restype = C.c_float
        fm.argtypes = [C.POINTER(C.c_float)]
        smax = fm(_ptr(c["F"]))
        rec("strain", i, U=U6, S=S2, Vt=Vt4, deda=deda, d2=d2, f=f6, h=h36, k=[k], smax=[smax])
    for i, c in enumerate(gen_ccd(rng, n)):
        ov = np.zeros(1, np.int32)
        f = fn("ccd")
        f.restype = C.c_float
        f.argtypes = [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float,
                      C.c_float, C.c_float, C.c_float, C.POINTER(C.c_int)]
        t = f(c["kind"], _ptr(c["x0"]), _ptr(c["x1"]), c["off"], c["ghat"], c["max_t"],
              c["eps"], _iptr(ov))
        rec("ccd", i, toi=[t], overlap=[float(ov[0])])
    for i, c in enumerate(gen_isect(rng, n)):
        f = fn("edge_triangle")
        f.restype = C.c_int
        r = f(_ptr(c["e"][0]), _ptr(c["e"][1]), _ptr(c["t"][0]), _ptr(c["t"][1]), _ptr(c["t"][2]))
        rec("isect", i, hit=[float(r)])
    for i, c in enumerate(gen_rod(rng, n)):
        g6, h36 = np.zeros(6, f32), np.zeros(36, f32)
        f = fn("hook")
        f.argtypes = [C.POINTER(C.c_float)] * 2 + [C.c_float] * 2 + [C.POINTER(C.c_float)] * 2
        f(_ptr(c["x0"]), _ptr(c["x1"]), c["l0"], c["w"], _ptr(g6), _ptr(h36))
        f9, h81 = np.zeros(9, f32), np.zeros(81, f32)
        f = fn("strand")
        f.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_float] + [C.POINTER(C.c_float)] * 2
        bx = np.ascontiguousarray(c["b"])
        f(_ptr(bx[0]), _ptr(bx[1]), _ptr(bx[2]), c["rest"], _ptr(f9), _ptr(h81))
        rec("rod", i, stretch_g=g6, stretch_h=h36, bend_f=f9, bend_h=h81)
    for i, c in enumerate(gen_solid(rng, n)):
        ft = fn("model_table")
        ft.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), C.c_float, C.c_float,
                       C.POINTER(C.c_float), C.POINTER(C.c_float)]
        d2a, d2b = np.zeros(2, f32), np.zeros(4, f32)
        ft(c["model"], 2, _ptr(c["a3"]), c["mu"], c["lmd"], _ptr(d2a), _ptr(d2b))
        d3a, d3b = np.zeros(3, f32), np.zeros(9, f32)
        ft(c["model"], 3, _ptr(c["a3"]), c["mu"], c["lmd"], _ptr(d3a), _ptr(d3b))
        U9, S3, Vt9 = np.zeros(9, f32), np.zeros(3, f32), np.zeros(9, f32)
        fn("svd33")(_ptr(c["F"]), _ptr(U9), _ptr(S3), _ptr(Vt9))
        f12, h144 = np.zeros(12, f32), np.zeros(144, f32)
        f = fn("tet")
        f.argtypes = [C.POINTER(C.c_float)] * 2 + [C.c_int] + [C.c_float] * 4 + [C.POINTER(C.c_float)] * 2
        f(_ptr(c["x"]), _ptr(c["inv"]), c["model"], c["mu"], c["lmd"], c["mass"], f32(1e-4),
          _ptr(f12), _ptr(h144))
        f9, h81 = np.zeros(9, f32), np.zeros(81, f32)
        f = fn("shell_model")
        f.argtypes = [C.POINTER(C.c_float)] * 2 + [C.c_int] + [C.c_float] * 4 + [C.POINTER(C.c_float)] * 2
        f(_ptr(c["tri"]), _ptr(c["inv2"]), c["model"], c["mu"], c["lmd"], c["mass"], f32(1e-4),
          _ptr(f9), _ptr(h81))
        rec("solid", i, table2_g=d2a, table2_h=d2b, table3_g=d3a, table3_h=d3b, svd_U=U9,
            svd_S=S3, svd_Vt=Vt9, tet_f=f12, tet_h=h144, shell_f=f9, shell_h=h81)
    return {k: np.stack(v) for k, v in res.items()}


# Relative tolerance (scaled by the case's largest magnitude) per output.
EXACT = {"isect.hit", "ccd.overlap"}
TOL = {
    "ccd.toi": 1e-5,
    "eig.vec3": 2e-3,   # eigenvectors of (near-)degenerate triples
    "eig.val3": 1e-5,
    "hinge.h": 2e-4,
    "hinge.f": 1e-4,
    "bw.shear_h": 1e-4,
    "bw.stretch_h": 1e-5,
    "strain.h": 1e-4,
}
DEFAULT_TOL = 2e-6
