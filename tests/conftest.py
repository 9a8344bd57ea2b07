import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "ppf-contact-solver_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)

# A fatal error inside the library returns a failed result to this process
# instead of exiting it (the reference driver's exit(1) behaviour is the
# default for every other host).
os.environ.setdefault("PPF_RETURN_ON_FATAL", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def product_lib():
    from ppf_gb300 import _lib, build

    build.build_product()
    return _lib.product()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import binding
    from ppf_gb300 import build

    build.build_oracle()
    return binding.oracle()


@pytest.fixture(scope="session")
def ref_lib():
    from oracle import binding
    from ppf_gb300 import build

    try:
        build.build_reference()
    except Exception:
        pass
    lib = binding.reference()
    if lib is None:
        pytest.skip("reference sources not present on this host")
    return lib


@pytest.fixture(scope="session")
def ref_pipeline_or_none():
    """The reference's own pipeline compiled as host code, or None where its
    sources are absent (the frozen fixtures stand in there)."""
    from oracle import binding
    from ppf_gb300 import build

    try:
        build.build_reference()
    except Exception:
        pass
    return binding.reference_pipeline()


@pytest.fixture
def rng():
    return np.random.default_rng(1234)


@pytest.fixture(autouse=True)
def _block_jacobi_after_each_test(request):
    """The library keeps its preconditioner choice across sessions (it is a
    process-wide setting, like the rest of its state): put block-Jacobi, the
    reference's, back after every GPU test, so no test inherits another's
    (the same for the PCG team and the iteration graph)."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    import ctypes

    from ppf_gb300 import _lib

    if _lib._PRODUCT is not None:
        _lib._PRODUCT.ppf_set_preconditioner(ctypes.c_int(0), ctypes.c_float(0.0))
        # and the default PCG team and Newton-iteration graph
        _lib._PRODUCT.ppf_set_pcg_team(ctypes.c_int(-1))
        _lib._PRODUCT.ppf_set_pcg_cta_threads(ctypes.c_uint(0))
        _lib._PRODUCT.ppf_set_iteration_graph(ctypes.c_int(1))
