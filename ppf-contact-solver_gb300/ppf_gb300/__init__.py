"""Host side of the GB300-native per-step contact solve.

The compute path is libppf_gb300.so (sm_103a CUDA + C ABI, see
include/ppf_gb300.h); this package builds it, binds it with ctypes, and
generates the seeded synthetic scenes the tests and the benchmark run.
"""
import os

# Many scenes stepped together run one stream each; with the CUDA default of
# 8 hardware work queues, streams beyond 8 share queues and their kernels
# wait on each other's. The count is read when the CUDA context is created,
# so it is set before anything in the process touches CUDA (a value already
# in the environment is kept).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import build  # noqa: F401,E402
from ._lib import LibraryMissing, product  # noqa: F401,E402
