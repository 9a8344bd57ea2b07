"""Builds the sm_103a library, the host scene builder and the CPU oracle.

Everything is compiled in-tree with nvcc / g++ directly (no cmake), one
translation unit per process in parallel, so a build on a 16-core host takes
well under a minute:

* ``ppf-contact-solver_gb300/lib/libppf_gb300.so`` -- the product: CUDA
  kernels for sm_103a plus the C ABI (``include/ppf_gb300.h``).
* ``oracle/liboracle_ppf.so`` -- the CPU oracle (test infrastructure only).
* ``oracle/_ref/libppfref.so`` -- the reference's own header-only element math
  compiled from its sources, built only where those sources are present.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parents[1]
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
PRODUCT_LIB = LIBDIR / "libppf_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle_ppf.so"
REF_LIB = ORACLE_DIR / "_ref" / "libppfref.so"
REF_PIPE_LIB = ORACLE_DIR / "_ref" / "libppfref_pipe.so"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
# -fmad=false: every single-precision operation rounds on its own, so the
# kernels compute the same bits as the CPU oracle built with
# -ffp-contract=off. Where the reference's contraction is part of the
# arithmetic (the swept leaf box), the kernels call fmaf explicitly. Host
# code of the CUDA sources is not contracted either.
NVCC_FLAGS = [
    "-std=c++17", "-O3", "-lineinfo", GENCODE, "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
    "-Xptxas", "-warn-spills",
]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off"]


def _sources(pattern_dirs, exts):
    out = []
    for d in pattern_dirs:
        for p in sorted(d.rglob("*")):
            if p.suffix in exts:
                out.append(p)
    return out


def _newest(paths):
    return max((p.stat().st_mtime for p in paths), default=0.0)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(
            "command failed:\n  " + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr
        )
    return r.stdout + r.stderr


def _jobs():
    return max(1, min(16, os.cpu_count() or 4))


def build_product(force: bool = False, verbose: bool = False) -> Path:
    """Compile csrc/gpu/*.cu and csrc/host/*.cpp into libppf_gb300.so."""
    cu = _sources([CSRC / "gpu"], {".cu"})
    cpp = _sources([CSRC / "host"], {".cpp"})
    deps = _sources([CSRC, INCLUDE], {".cu", ".cuh", ".cpp", ".h", ".hpp"})
    if not force and PRODUCT_LIB.exists() and PRODUCT_LIB.stat().st_mtime > _newest(deps):
        return PRODUCT_LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    jobs = []
    for src in cu:
        obj = BUILD / (src.stem + ".cu.o")
        jobs.append([NVCC, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = BUILD / (src.stem + ".cpp.o")
        jobs.append([CXX, *CXX_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(_jobs()) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    objs = [str(BUILD / (s.stem + ".cu.o")) for s in cu] + [
        str(BUILD / (s.stem + ".cpp.o")) for s in cpp
    ]
    tmp = PRODUCT_LIB.with_suffix(".so.tmp")
    _run([NVCC, GENCODE, "-shared", "-o", str(tmp), *objs, "-lcudart"])
    os.replace(tmp, PRODUCT_LIB)
    return PRODUCT_LIB


DRIVER = PKG / "bin" / "ppf-contact-solver"


def build_driver(force: bool = False) -> Path:
    """Compile the solver executable (csrc/driver/main.cpp) against the
    product library, with an rpath to it."""
    srcs = _sources([CSRC / "driver"], {".cpp"})
    deps = srcs + _sources([INCLUDE], {".h"}) + [PRODUCT_LIB]
    if not force and DRIVER.exists() and DRIVER.stat().st_mtime > _newest(deps):
        return DRIVER
    DRIVER.parent.mkdir(parents=True, exist_ok=True)
    tmp = DRIVER.with_suffix(".tmp")
    _run([CXX, "-std=c++17", "-O2", "-I", str(INCLUDE), *map(str, srcs), "-o", str(tmp),
          "-L", str(LIBDIR), "-lppf_gb300", "-Wl,-rpath,$ORIGIN/../lib"])
    os.replace(tmp, DRIVER)
    return DRIVER


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle (oracle/*.cpp) into oracle/liboracle_ppf.so."""
    srcs = sorted(ORACLE_DIR.glob("oracle_*.cpp"))
    deps = srcs + sorted(ORACLE_DIR.glob("*.h")) + _sources(
        [CSRC / "physics", INCLUDE], {".cuh", ".h"})
    if not force and ORACLE_LIB.exists() and ORACLE_LIB.stat().st_mtime > _newest(deps):
        return ORACLE_LIB
    obj_dir = ORACLE_DIR / "_build"
    obj_dir.mkdir(exist_ok=True)
    jobs = []
    for s in srcs:
        jobs.append([CXX, *CXX_FLAGS, "-fopenmp", "-I", str(INCLUDE), "-c", str(s),
                     "-o", str(obj_dir / (s.stem + ".o"))])
    with cf.ThreadPoolExecutor(_jobs()) as ex:
        list(ex.map(_run, jobs))
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    _run([CXX, "-shared", "-fopenmp", "-o", str(tmp),
          *[str(obj_dir / (s.stem + ".o")) for s in srcs]])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_root() -> Path:
    """The reference checkout: $PPF_REF_ROOT, else a ``reference`` directory
    beside this repository's root."""
    env = os.environ.get("PPF_REF_ROOT")
    return Path(env) if env else ROOT.parent / "reference"


def build_reference(force: bool = False) -> Path | None:
    """Compile the reference's header-only element math where its sources are
    present (oracle/Makefile); returns None when they are not."""
    ref_root = reference_root()
    if not (ref_root / "crates/ppf-cts-solver/src/cpp/data.hpp").exists():
        return None
    if shutil.which("make") is None:
        return None
    args = ["make", "-C", str(ORACLE_DIR), f"REF_ROOT={ref_root}", "ref"]
    if force:
        args.insert(1, "-B")
    _run(args)
    return REF_LIB


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(3) as ex:
        f1 = ex.submit(build_product, force)
        f2 = ex.submit(build_oracle, force)
        f3 = ex.submit(build_reference, force)
        f1.result()
        f2.result()
        f3.result()
    build_driver(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", PRODUCT_LIB, ORACLE_LIB)
