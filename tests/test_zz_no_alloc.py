"""The allocation-free radix sort (ppf_radix_sort_device_noalloc) against the
allocating one (ppf_radix_sort_device) on the same device data.

Integer work, so the comparison is bit-exact. Two calls in a row reuse the
same static scratch. A size above the stated limit is rejected without
touching the data. This file sorts last in collection order; it also passes
on its own.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 20  # PPF_NOALLOC_SORT_MAX_PAIRS


@pytest.fixture(scope="module")
def lib(product_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    product_lib.ppf_radix_sort_device_noalloc.restype = C.c_int
    product_lib.ppf_radix_sort_device_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_uint,
                                                          C.c_int, C.c_void_p]
    return product_lib


def _sort_both(lib, keys, vals, bits):
    import torch

    stream = torch.cuda.current_stream().cuda_stream
    ka = torch.from_numpy(keys.view(np.int32)).cuda()
    va = torch.from_numpy(vals.view(np.int32)).cuda()
    kb, vb = ka.clone(), va.clone()
    n = keys.size
    rc_a = lib.ppf_radix_sort_device(ka.data_ptr(), va.data_ptr(), n, bits, stream)
    rc_b = lib.ppf_radix_sort_device_noalloc(kb.data_ptr(), vb.data_ptr(), n, bits, stream)
    torch.cuda.synchronize()
    return (rc_a, rc_b, ka.cpu().numpy().view(np.uint32), va.cpu().numpy().view(np.uint32),
            kb.cpu().numpy().view(np.uint32), vb.cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("n,bits", [(LIMIT, 30), (300_001, 24)])
def test_noalloc_matches_allocating_sort_twice(lib, n, bits):
    rng = np.random.default_rng(n)
    for call in range(2):
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint32)
        keys[: n // 7] = keys[n // 3]  # runs of equal keys: stability matters
        vals = np.arange(n, dtype=np.uint32)
        rc_a, rc_b, ka, va, kb, vb = _sort_both(lib, keys, vals, bits)
        assert rc_a == 0 and rc_b == 0, (call, rc_a, rc_b)
        assert np.array_equal(kb, ka), call
        assert np.array_equal(vb, va), call
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(vb, order.astype(np.uint32)), call


def test_noalloc_rejects_above_limit(lib):
    import torch

    n = LIMIT + 1
    keys = torch.arange(n, 0, -1, dtype=torch.int32, device="cuda")
    vals = torch.zeros(n, dtype=torch.int32, device="cuda")
    before = keys.clone()
    rc = lib.ppf_radix_sort_device_noalloc(keys.data_ptr(), vals.data_ptr(), n, 30,
                                           torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == -2
    assert torch.equal(keys, before)
