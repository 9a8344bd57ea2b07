"""Host side of the GB300-native per-step contact solve.

The compute path is libppf_gb300.so (sm_103a CUDA + C ABI, see
include/ppf_gb300.h); this package builds it, binds it with ctypes, and
generates the seeded synthetic scenes the tests and the benchmark run.
"""
from . import build  # noqa: F401
from ._lib import LibraryMissing, product  # noqa: F401
