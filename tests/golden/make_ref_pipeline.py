"""Freezes the reference's own Newton-system assembly, line searches and
intersection checks on the two-sheets scene, and its assembly and rod
strain-limit line search on the rods-and-sheet scene (ref_rods.npz), and its
assembly on the solids-and-sheet scene (ref_solids.npz) and the stitched
sheets (ref_stitches.npz).

Builds oracle/_ref/libppfref_pipe.so from the reference sources
(oracle/Makefile), drives it through the states of
tests/ref_pipeline_cases.py (the oracle's step loop supplies the states) and
writes tests/golden/ref_pipeline.npz. Run from the repository root:

    python tests/golden/make_ref_pipeline.py
"""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT / "tests", ROOT / "ppf-contact-solver_gb300", ROOT):
    sys.path.insert(0, str(p))

import ref_pipeline_cases as rpc  # noqa: E402
import step_scenes  # noqa: E402
from oracle import binding  # noqa: E402
from ppf_gb300 import build  # noqa: E402


def main():
    if build.build_reference(force=True) is None:
        raise SystemExit("reference sources not found")
    ref = binding.reference_pipeline()
    sc, _ = step_scenes.two_sheets()
    o = binding.OracleSession(sc)
    assert ref.refpipe_init(sc.dataset, C.byref(o.param))
    # the first Newton system at the scene's start state (later states
    # depend on the oracle's own trajectory and are compared live)
    curr, prev, prm, target, dt, *_ = rpc.oracle_first_system(o)
    keys, blocks, force, count = rpc.reference_first_system(ref, curr, prev, prm, target, dt)
    out = {"keys": keys, "blocks": blocks.astype(np.float32), "force": force,
           "contacts": np.uint32(count)}
    # line searches and intersection checks from the start state
    _, dx, _, _ = o.newton_system()
    out["ls_dx"] = dx.reshape(-1).astype(np.float32)
    for name, x1 in rpc.line_search_cases(curr, dx).items():
        pin, ov = C.c_uint(), C.c_int()
        toi = ref.refpipe_line_search(curr, x1, C.byref(pin), C.byref(ov))
        out[f"ls_{name}"] = np.array([toi, ref.refpipe_strain_line_search(curr, x1)], np.float32)
        out[f"ls_{name}_flags"] = np.array([pin.value, ov.value], np.uint32)
    for name, x in rpc.intersection_cases(curr).items():
        out[f"isect_{name}"] = np.uint8(ref.refpipe_check_intersection(x))
    path = Path(__file__).parent / "ref_pipeline.npz"
    np.savez_compressed(path, **out)
    print("wrote", len(out), "arrays,", path.stat().st_size, "bytes")
    rods(ref)
    for name, make in (("solids", step_scenes.solids_and_sheet),
                       ("stitches", step_scenes.stitched_sheets)):
        sc, _ = make()
        out = first_system(ref, sc)
        path = Path(__file__).parent / f"ref_{name}.npz"
        np.savez_compressed(path, **out)
        print("wrote", len(out), "arrays,", path.stat().st_size, "bytes",
              "contacts", int(out["contacts"]))


def first_system(ref, sc):
    """A scene's first Newton system at its start state as the reference
    assembles it: the solids-and-sheet scene (ARAP and SNHk tets with
    damping, an StVK sheet, contact on the solids' boundary faces) and the
    stitched sheets (vertex-to-face and vertex-to-vertex stitches)."""
    prm = sc.param.contents
    assert ref.refpipe_init(sc.dataset, C.byref(prm))
    curr, prev = rpc.dataset_positions(sc)
    target = rpc.step_target(sc, curr, prev)
    dt = float(np.float32(prm.dt) * np.float32(prm.playback))
    keys, blocks, force, count = rpc.reference_first_system(ref, curr, prev, prm, target, dt)
    return {"keys": keys, "blocks": blocks.astype(np.float32), "force": force,
            "contacts": np.uint32(count), "target": target}


def rods(ref):
    """The rods-and-sheet scene's first Newton system at its start state, as
    the reference assembles it (rod stretch, bending and strain limit with
    damping, shell membrane and bending with damping, contact), and the rod
    strain-limit line search toward a 3 % stretch of rod A."""
    sc, info = step_scenes.rods_and_sheet()
    prm = sc.param.contents
    assert ref.refpipe_init(sc.dataset, C.byref(prm))
    curr, prev = rpc.dataset_positions(sc)
    target = rpc.step_target(sc, curr, prev)
    dt = float(np.float32(prm.dt) * np.float32(prm.playback))
    keys, blocks, force, count = rpc.reference_first_system(ref, curr, prev, prm, target, dt)
    out = {"keys": keys, "blocks": blocks.astype(np.float32), "force": force,
           "contacts": np.uint32(count), "target": target}
    a0, na = info["rod_a"]
    x1 = curr.reshape(-1, 3).copy()
    c = x1[a0:a0 + na].mean(axis=0)
    x1[a0:a0 + na] = c + 1.03 * (x1[a0:a0 + na] - c)
    x1 = x1.reshape(-1).astype(np.float32)
    out["rod_ls"] = np.array([ref.refpipe_rod_strain_line_search(curr, x1)], np.float32)
    out["rod_ls_x1"] = x1
    path = Path(__file__).parent / "ref_rods.npz"
    np.savez_compressed(path, **out)
    print("wrote", len(out), "arrays,", path.stat().st_size, "bytes", "contacts", count)


if __name__ == "__main__":
    main()
