"""LBVH and radix-sort parity: the sm_103a kernels against the CPU oracle.

Bar: bit-exact (Morton codes, sort permutation, node array, leaf and internal
boxes). The oracle restates crates/ppf-cts-solver/src/cpp/lbvh/lbvh.cu and
kernels/radix_sort.cu; its own invariants are checked on the CPU below.
"""
import numpy as np
import pytest

from ppf_gb300 import _lib, meshes


def _cloth(rng, nx, ny, noise=0.02):
    v, f = meshes.grid(nx, ny)
    v = v + rng.normal(0, noise, v.shape).astype(np.float32)
    return v, f


def _prims(kind, f):
    if kind == 3:
        return f
    if kind == 2:
        return meshes.edges_of(f)
    return None


def _count(kind, v, f):
    if kind == 3:
        return len(f)
    if kind == 2:
        return len(meshes.edges_of(f))
    return len(v)


def _check_tree(root, node, box, n):
    """Structural invariants of an LBVH: every leaf reached once, children
    boxes inside parents, leaves hold a permutation of the primitives."""
    if n == 1:
        assert root == 0 and node[0, 0] == 1 and node[0, 1] == 0
        return
    assert root == n
    leaves = sorted(int(node[i, 0]) - 1 for i in range(n))
    assert leaves == list(range(n))
    seen = np.zeros(2 * n - 1, np.int32)
    stack = [root]
    while stack:
        i = stack.pop()
        seen[i] += 1
        if node[i, 1] == 0:
            continue
        for c in (node[i, 0] - 1, node[i, 1] - 1):
            assert np.all(box[i, :3] <= box[c, :3]) and np.all(box[i, 4:7] >= box[c, 4:7])
            stack.append(int(c))
    assert np.all(seen == 1)


@pytest.mark.parametrize("kind", [1, 2, 3])
def test_oracle_lbvh_invariants(oracle_lib, rng, kind):
    v, f = _cloth(rng, 17, 13)
    n = _count(kind, v, f)
    margin = rng.uniform(1e-4, 1e-3, n).astype(np.float32)
    root, node, box, keys = _lib.lbvh(oracle_lib.oracle_lbvh_build, kind, v, v,
                                      _prims(kind, f), margin)
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    _check_tree(root, node, box, n)


def test_oracle_stable_sort(oracle_lib, rng):
    n = 5000
    keys = rng.integers(0, 64, n).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = keys.copy(), vals.copy()
    oracle_lib.oracle_stable_sort(k, v, n, 32)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(v, vals[order]) and np.array_equal(k, keys[order])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 3, 255, 256, 2047, 2048, 2049, 100_000, 3_141_633])
def test_radix_sort_matches_stable_sort(product_lib, rng, n):
    keys = rng.integers(0, 1 << 30, n).astype(np.uint32)
    keys[: n // 3] = keys[0]  # long run of equal keys: stability matters
    vals = np.arange(n, dtype=np.uint32)
    k, v = keys.copy(), vals.copy()
    assert product_lib.ppf_radix_sort_host(k, v, n, 30) == 0
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order])
    assert np.array_equal(v, vals[order])


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [8, 16, 24, 32])
def test_radix_sort_key_bits(product_lib, rng, bits):
    n = 70_001
    hi = (1 << bits) if bits < 32 else (1 << 32)
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = keys.copy(), vals.copy()
    assert product_lib.ppf_radix_sort_host(k, v, n, bits) == 0
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(v, vals[order])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [1, 2, 3])
@pytest.mark.parametrize("shape", [(2, 2), (3, 2), (64, 64), (181, 97)])
def test_lbvh_bit_exact(product_lib, oracle_lib, rng, kind, shape):
    v, f = _cloth(rng, *shape)
    n = _count(kind, v, f)
    margin = rng.uniform(1e-4, 1e-3, n).astype(np.float32)
    v1 = v + rng.normal(0, 0.01, v.shape).astype(np.float32)
    p = _prims(kind, f)
    a = _lib.lbvh(product_lib.ppf_lbvh_build_host, kind, v, v1, p, margin, 1.25)
    b = _lib.lbvh(oracle_lib.oracle_lbvh_build, kind, v, v1, p, margin, 1.25)
    assert a[0] == b[0]
    assert np.array_equal(a[3], b[3]), "Morton codes / sort order differ"
    assert np.array_equal(a[1], b[1]), "node arrays differ"
    assert np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32)), "boxes differ"
    _check_tree(*a[:3], n)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [1, 2, 3])
def test_lbvh_single_primitive(product_lib, oracle_lib, kind):
    """One primitive: the tree is that leaf alone (root 0), its box the swept
    primitive's, as the oracle has it."""
    v = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], np.float32)
    v1 = v + np.float32(0.01)
    prims = {1: None, 2: np.array([[0, 1]], np.uint32), 3: np.array([[0, 1, 2]], np.uint32)}[kind]
    x0 = v[:1] if kind == 1 else v
    x1 = v1[:1] if kind == 1 else v1
    margin = np.full(1, 5e-4, np.float32)
    a = _lib.lbvh(product_lib.ppf_lbvh_build_host, kind, x0, x1, prims, margin, 1.0)
    b = _lib.lbvh(oracle_lib.oracle_lbvh_build, kind, x0, x1, prims, margin, 1.0)
    assert a[0] == b[0] == 0
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))


@pytest.mark.gpu
def test_radix_sort_empty_input(product_lib):
    keys = np.zeros(0, np.uint32)
    vals = np.zeros(0, np.uint32)
    assert product_lib.ppf_radix_sort_host(keys, vals, 0, 30) == 0


@pytest.mark.gpu
def test_lbvh_duplicate_centroids(product_lib, oracle_lib):
    """All primitives at one point: every Morton code ties, so the topology is
    decided by the index tie-break alone."""
    n = 1000
    v = np.zeros((n, 3), np.float32)
    margin = np.full(n, 5e-4, np.float32)
    a = _lib.lbvh(product_lib.ppf_lbvh_build_host, 1, v, v, None, margin)
    b = _lib.lbvh(oracle_lib.oracle_lbvh_build, 1, v, v, None, margin)
    assert np.array_equal(a[1], b[1])
    _check_tree(*a[:3], n)


@pytest.mark.gpu
def test_lbvh_large_face_tree(product_lib, oracle_lib, rng):
    """The 1024 x 1024 cloth's face tree (2,093,058 faces)."""
    v, f = meshes.grid(1024, 1024)
    v = v + rng.normal(0, 1e-3, v.shape).astype(np.float32)
    margin = np.full(len(f), 5e-4, np.float32)
    a = _lib.lbvh(product_lib.ppf_lbvh_build_host, 3, v, v, f, margin)
    b = _lib.lbvh(oracle_lib.oracle_lbvh_build, 3, v, v, f, margin)
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))
