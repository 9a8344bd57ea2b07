"""ctypes binding of libppf_gb300.so.

The library must be present: every entry point here goes through it, and a
missing library raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

_PRODUCT = None

u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


class LibraryMissing(RuntimeError):
    pass


def _opt(ptr_type):
    """ndpointer that also accepts None."""

    class _Opt(ptr_type):
        @classmethod
        def from_param(cls, obj):
            if obj is None:
                return None
            return super().from_param(obj)

    return _Opt


u32p_opt = _opt(u32p)
f32p_opt = _opt(f32p)


def product() -> C.CDLL:
    """The GB300 library. Raises LibraryMissing if it has not been built."""
    global _PRODUCT
    if _PRODUCT is None:
        path = Path(os.environ.get("PPF_GB300_LIB", _build.PRODUCT_LIB))
        if not path.exists():
            raise LibraryMissing(
                f"{path} is missing: run __graft_entry__.build() (the CUDA "
                "library is required; there is no CPU fallback)")
        lib = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
        _declare_product(lib)
        _PRODUCT = lib
    return _PRODUCT


def _declare_product(lib):
    lib.ppf_lbvh_build_host.restype = C.c_uint
    lib.ppf_lbvh_build_host.argtypes = [
        C.c_int, f32p, f32p, C.c_uint, u32p_opt, C.c_uint, f32p, C.c_float,
        u32p_opt, f32p_opt, u32p_opt]
    lib.ppf_radix_sort_host.restype = C.c_int
    lib.ppf_radix_sort_host.argtypes = [u32p, u32p, C.c_uint, C.c_int]
    lib.ppf_radix_sort_device.restype = C.c_int
    lib.ppf_radix_sort_device.argtypes = [C.c_void_p, C.c_void_p, C.c_uint,
                                          C.c_int, C.c_void_p]


def lbvh(fn, kind: int, x0, x1, prims, margin, extrapolate=1.0):
    """Runs one LBVH build through `fn`, a C function with the signature of
    ppf_lbvh_build_host, and returns (root, node[2n-1, 2], box[2n-1, 8],
    keys[n])."""
    x0 = np.ascontiguousarray(x0, np.float32).reshape(-1)
    x1 = np.ascontiguousarray(x1, np.float32).reshape(-1)
    n_verts = x0.size // 3
    margin = np.ascontiguousarray(margin, np.float32)
    n = margin.size
    if prims is not None:
        prims = np.ascontiguousarray(prims, np.uint32).reshape(-1)
    nn = max(2 * n - 1, 1)
    node = np.zeros(2 * nn, np.uint32)
    box = np.zeros(8 * nn, np.float32)
    keys = np.zeros(max(n, 1), np.uint32)
    root = fn(kind, x0, x1, n_verts, prims, n, margin, np.float32(extrapolate),
              node, box, keys)
    return root, node.reshape(nn, 2), box.reshape(nn, 8), keys[:n]
