"""Seeded synthetic meshes (cloth grids, tubes, boxes) used by the scenes."""
from __future__ import annotations

import numpy as np


def grid(nx: int, ny: int, size_x: float = 1.0, size_y: float = 1.0):
    """nx x ny vertex grid on [-sx/2, sx/2] x [-sy/2, sy/2] in the XZ plane
    (y = 0), split into triangles along alternating diagonals.
    Returns (vertices [n,3] f32, faces [f,3] u32)."""
    xs = np.linspace(-0.5 * size_x, 0.5 * size_x, nx, dtype=np.float64)
    zs = np.linspace(-0.5 * size_y, 0.5 * size_y, ny, dtype=np.float64)
    X, Z = np.meshgrid(xs, zs, indexing="xy")  # [ny, nx]
    v = np.stack([X.ravel(), np.zeros(X.size), Z.ravel()], axis=1).astype(np.float32)
    J, I = np.meshgrid(np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    a = (J * nx + I).ravel()
    b, c = a + 1, a + nx
    d = c + 1
    even = ((I + J) % 2 == 0).ravel()
    t0 = np.where(even[:, None], np.stack([a, c, b], 1), np.stack([a, c, d], 1))
    t1 = np.where(even[:, None], np.stack([b, c, d], 1), np.stack([a, d, b], 1))
    faces = np.stack([t0, t1], 1).reshape(-1, 3)
    return v, faces.astype(np.uint32)


def tube(n_around: int, n_along: int, radius: float, length: float):
    """Open cylinder along x: n_around x n_along vertices."""
    th = np.linspace(0.0, 2.0 * np.pi, n_around, endpoint=False)
    xs = np.linspace(-0.5 * length, 0.5 * length, n_along)
    v = np.zeros((n_along, n_around, 3), np.float64)
    v[:, :, 0] = xs[:, None]
    v[:, :, 1] = radius * np.cos(th)[None, :]
    v[:, :, 2] = radius * np.sin(th)[None, :]
    v = v.reshape(-1, 3)
    J, I = np.meshgrid(np.arange(n_along - 1), np.arange(n_around), indexing="ij")
    a = (J * n_around + I).ravel()
    b = (J * n_around + (I + 1) % n_around).ravel()
    c, d = a + n_around, b + n_around
    faces = np.stack([np.stack([a, c, b], 1), np.stack([b, c, d], 1)], 1).reshape(-1, 3)
    return v.astype(np.float32), faces.astype(np.uint32)


def box(side: float, center=(0.0, 0.0, 0.0)):
    """Closed axis-aligned cube, 8 vertices / 12 outward-facing triangles."""
    h = 0.5 * side
    c = np.asarray(center, np.float64)
    v = np.array([[-h, -h, -h], [h, -h, -h], [h, h, -h], [-h, h, -h],
                  [-h, -h, h], [h, -h, h], [h, h, h], [-h, h, h]]) + c
    f = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5],
                  [0, 5, 4], [2, 3, 7], [2, 7, 6], [1, 2, 6], [1, 6, 5],
                  [0, 4, 7], [0, 7, 3]], np.uint32)
    return v.astype(np.float32), f


def tet_box(n: int, side: float, center=(0.0, 0.0, 0.0)):
    """Solid cube of (n+1)^3 vertices, each of its n^3 cells split into six
    tets along the main diagonal (one per axis order), all positively
    oriented. Returns (vertices [(n+1)^3, 3] f32, tets [6 n^3, 4] u32)."""
    g = np.linspace(-0.5 * side, 0.5 * side, n + 1)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    v = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) + np.asarray(center, np.float64)
    idx = np.arange((n + 1) ** 3).reshape(n + 1, n + 1, n + 1)
    unit = np.eye(3, dtype=int)
    orders = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    tets = []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                c = np.array([i, j, k])
                for o in orders:
                    p1 = c + unit[o[0]]
                    p2 = p1 + unit[o[1]]
                    t = [idx[tuple(c)], idx[tuple(p1)], idx[tuple(p2)], idx[tuple(c + 1)]]
                    d = np.linalg.det(np.stack([v[t[1]] - v[t[0]], v[t[2]] - v[t[0]],
                                                v[t[3]] - v[t[0]]], 1))
                    if d < 0:
                        t[1], t[2] = t[2], t[1]
                    tets.append(t)
    return v.astype(np.float32), np.asarray(tets, np.uint32)


def edges_of(faces: np.ndarray) -> np.ndarray:
    """Unique undirected edges in first-seen order (face order, then corner
    order j -> j+1), each as (first-seen endpoint, next endpoint)."""
    seen = {}
    out = []
    for f in faces:
        for j in range(3):
            a, b = int(f[j]), int(f[(j + 1) % 3])
            key = (a, b) if a < b else (b, a)
            if key not in seen:
                seen[key] = len(out)
                out.append((a, b))
    return np.asarray(out, np.uint32).reshape(-1, 2)
