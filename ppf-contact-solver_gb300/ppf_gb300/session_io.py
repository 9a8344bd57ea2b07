"""Scene directories in the reference's on-disk session format, for the
solver executable (csrc/driver/main.cpp).

`write_session` writes the subset of the layout the reference's frontend
exports (frontend/_scene_.py:806-1000, read back by crates/ppf-cts-solver/
src/scene.rs:443-1110) that this library simulates: shells with per-face
materials, rods with per-rod materials, stitches, fix and pull pins without
operations, one-keyframe walls and
spheres, and a static collision mesh; info.toml and param.toml as the
frontend writes them. `read_frame` reads a vert_<n>.bin the executable
wrote.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import build as _build


@dataclass
class Wall:
    position: tuple
    normal: tuple = (0.0, 1.0, 0.0)
    contact_gap: float = 1e-3
    friction: float = 0.0


@dataclass
class Sphere:
    center: tuple
    radius: float
    contact_gap: float = 1e-3
    friction: float = 0.0
    invert: bool = False
    hemisphere: bool = False


@dataclass
class SessionScene:
    vert: np.ndarray                     # (n, 3) positions
    tri: np.ndarray                      # (F, 3) vertex indices
    face_params: dict                    # name -> (F,) float32, e.g. "young-mod"
    vel: np.ndarray | None = None        # (n, 3)
    pins: list = field(default_factory=list)   # (indices, pull weight) pairs
    walls: list = field(default_factory=list)
    spheres: list = field(default_factory=list)
    static_vert: np.ndarray | None = None
    static_tri: np.ndarray | None = None
    static_params: dict = field(default_factory=dict)  # name -> (Fs,) float32
    param: dict = field(default_factory=dict)          # [param] keys of param.toml
    rod: np.ndarray | None = None        # (R, 2) vertex indices of rod edges
    rod_params: dict = field(default_factory=dict)     # name -> (R,) float32, e.g. "bend"
    stitch_ind: np.ndarray | None = None  # (M, 6) vertex indices
    stitch_w: np.ndarray | None = None    # (M, 6) barycentric weights
    stitch_stiffness: np.ndarray | None = None  # (M,)


def _toml_value(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, str):
        return f'"{v}"'
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(_toml_value(x) for x in v) + "]"
    return repr(float(v)) if isinstance(v, float) else str(v)


def write_session(path, sc: SessionScene) -> Path:
    path = Path(path)
    b = path / "bin"
    (b / "param").mkdir(parents=True, exist_ok=True)
    n, nf = len(sc.vert), len(sc.tri)
    nr = 0 if sc.rod is None else len(sc.rod)
    n_seam = 0 if sc.stitch_ind is None else len(sc.stitch_ind)
    ns = 0 if sc.static_vert is None else len(sc.static_vert)
    nst = 0 if sc.static_tri is None else len(sc.static_tri)
    lines = ["[count]", f"vert = {n}", f"rod = {nr}", f"tri = {nf}", "tet = 0",
             f"static_vert = {ns}", f"static_tri = {nst}", f"pin_block = {len(sc.pins)}",
             f"wall = {len(sc.walls)}", f"sphere = {len(sc.spheres)}", f"stitch = {n_seam}",
             "rod_vert_start = 0", "rod_vert_end = 0", "shell_vert_start = 0",
             f"shell_vert_end = {n}", "rod_count = 0", "shell_count = 1", ""]
    for i, (ind, pull) in enumerate(sc.pins):
        lines += [f"[pin-{i}]", f"pin = {len(ind)}", "operation_count = 0",
                  f"pull = {float(pull)}", ""]
        np.asarray(ind, np.uint64).tofile(b / f"pin-ind-{i}.bin")
    for i, w in enumerate(sc.walls):
        lines += [f"[wall-{i}]", "keyframe = 1", f"nx = {float(w.normal[0])}",
                  f"ny = {float(w.normal[1])}", f"nz = {float(w.normal[2])}",
                  'transition = "linear"', f"contact-gap = {float(w.contact_gap)}",
                  f"friction = {float(w.friction)}", ""]
        np.asarray(w.position, np.float64).reshape(1, 3).tofile(b / f"wall-pos-{i}.bin")
        np.zeros(1, np.float64).tofile(b / f"wall-timing-{i}.bin")
    for i, s in enumerate(sc.spheres):
        lines += [f"[sphere-{i}]", f"invert = {_toml_value(s.invert)}",
                  f"hemisphere = {_toml_value(s.hemisphere)}", 'transition = "linear"',
                  "keyframe = 1", f"contact-gap = {float(s.contact_gap)}",
                  f"friction = {float(s.friction)}", ""]
        np.asarray(s.center, np.float64).reshape(1, 3).tofile(b / f"sphere-pos-{i}.bin")
        np.asarray([s.radius], np.float32).tofile(b / f"sphere-radius-{i}.bin")
        np.zeros(1, np.float64).tofile(b / f"sphere-timing-{i}.bin")
    (path / "info.toml").write_text("\n".join(lines) + "\n", encoding="utf-8")
    prm = ["[param]"] + [f"{k} = {_toml_value(v)}" for k, v in sc.param.items()]
    (path / "param.toml").write_text("\n".join(prm) + "\n", encoding="utf-8")
    np.zeros((1, 3), np.float64).tofile(b / "displacement.bin")
    np.zeros(n, np.uint32).tofile(b / "vert_dmap.bin")
    np.asarray(sc.vert, np.float64).tofile(b / "vert.bin")
    vel = np.zeros((n, 3), np.float32) if sc.vel is None else np.asarray(sc.vel, np.float32)
    vel.tofile(b / "vel.bin")
    np.asarray(sc.tri, np.uint64).tofile(b / "tri.bin")
    for k, v in sc.face_params.items():
        if k == "model":
            np.asarray(v, np.uint8).tofile(b / "param" / "tri-model.bin")
        else:
            np.asarray(v, np.float32).tofile(b / "param" / f"tri-{k}.bin")
    if n_seam:
        np.asarray(sc.stitch_ind, np.uint64).tofile(b / "stitch_ind.bin")
        np.asarray(sc.stitch_w, np.float32).tofile(b / "stitch_w.bin")
        if sc.stitch_stiffness is not None:
            np.asarray(sc.stitch_stiffness, np.float32).tofile(b / "stitch_stiffness.bin")
    if nr:
        np.asarray(sc.rod, np.uint64).tofile(b / "rod.bin")
        for k, v in sc.rod_params.items():
            np.asarray(v, np.float32).tofile(b / "param" / f"rod-{k}.bin")
    if ns:
        np.asarray(sc.static_vert, np.float64).tofile(b / "static_vert.bin")
        np.zeros(ns, np.uint32).tofile(b / "static_vert_dmap.bin")
        np.asarray(sc.static_tri, np.uint64).tofile(b / "static_tri.bin")
        for k, v in sc.static_params.items():
            np.asarray(v, np.float32).tofile(b / "param" / f"static-{k}.bin")
    return path


def read_frame(output, frame: int) -> np.ndarray:
    return np.fromfile(Path(output) / f"vert_{frame}.bin", np.float32).reshape(-1, 3)


def executable() -> Path:
    """The solver executable, built with the library."""
    return _build.DRIVER
