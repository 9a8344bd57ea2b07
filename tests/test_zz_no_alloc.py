"""The allocation-free radix sort (ppf_radix_sort_device_noalloc) against the
allocating one (ppf_radix_sort_device) on the same device data.

The entry point is for callers that cannot allocate device memory at the
point of the call: a per-frame loop where a cudaMalloc / cudaFree would
synchronize the device, or a host whose own allocator owns the device
memory. So besides the sort's result this file checks what it exists for:
after one warm-up call (n = 0, which performs the per-device set-up), more
calls leave the device's free memory unchanged.

Integer work, so the comparison is bit-exact. Two calls in a row reuse the
same static scratch, and the status word reads 0 after each. A size above
the stated limit is rejected without touching the data. This file sorts
last in collection order; it also passes on its own in a fresh process.
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
    for name in ("ppf_radix_sort_noalloc_status", "ppf_radix_sort_device_status"):
        getattr(product_lib, name).restype = C.c_int
        getattr(product_lib, name).argtypes = [C.c_void_p]
    stream = torch.cuda.current_stream().cuda_stream
    # warm-up: the per-device set-up, with nothing to sort
    assert product_lib.ppf_radix_sort_device_noalloc(None, None, 0, 30, stream) == 0
    assert product_lib.ppf_radix_sort_noalloc_status(stream) == 0
    return product_lib


def _sort_both(lib, keys, vals, bits):
    import torch

    stream = torch.cuda.current_stream().cuda_stream
    ka = torch.from_numpy(keys.view(np.int32)).cuda()
    va = torch.from_numpy(vals.view(np.int32)).cuda()
    kb, vb = ka.clone(), va.clone()
    n = keys.size
    rc_a = lib.ppf_radix_sort_device(ka.data_ptr(), va.data_ptr(), n, bits, stream)
    st_a = lib.ppf_radix_sort_device_status(stream)
    rc_b = lib.ppf_radix_sort_device_noalloc(kb.data_ptr(), vb.data_ptr(), n, bits, stream)
    st_b = lib.ppf_radix_sort_noalloc_status(stream)
    torch.cuda.synchronize()
    return (rc_a, rc_b, st_a, st_b, ka.cpu().numpy().view(np.uint32),
            va.cpu().numpy().view(np.uint32), kb.cpu().numpy().view(np.uint32),
            vb.cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("n,bits", [(LIMIT, 30), (300_001, 24)])
def test_noalloc_matches_allocating_sort_twice(lib, n, bits):
    rng = np.random.default_rng(n)
    for call in range(2):
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint32)
        keys[: n // 7] = keys[n // 3]  # runs of equal keys: stability matters
        vals = np.arange(n, dtype=np.uint32)
        rc_a, rc_b, st_a, st_b, ka, va, kb, vb = _sort_both(lib, keys, vals, bits)
        assert rc_a == 0 and rc_b == 0, (call, rc_a, rc_b)
        assert st_a == 0 and st_b == 0, (call, st_a, st_b)
        assert np.array_equal(kb, ka), call
        assert np.array_equal(vb, va), call
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(vb, order.astype(np.uint32)), call


def test_noalloc_calls_leave_free_memory_unchanged(lib):
    import torch

    stream = torch.cuda.current_stream().cuda_stream
    n = 500_000
    rng = np.random.default_rng(7)
    keys = torch.from_numpy(rng.integers(0, 1 << 30, n, dtype=np.uint32).view(np.int32)).cuda()
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    assert lib.ppf_radix_sort_device_noalloc(keys.data_ptr(), vals.data_ptr(), n, 30, stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert lib.ppf_radix_sort_device_noalloc(keys.data_ptr(), vals.data_ptr(), n, 30,
                                                 stream) == 0
        assert lib.ppf_radix_sort_noalloc_status(stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    k = keys.cpu().numpy().view(np.uint32)
    assert np.all(k[1:] >= k[:-1])


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
