"""The sample-offset pass's reference-shaped trees (csrc/reftree.cpp) built with
their threaded top levels have exactly the layout of the sequential build
(nodes, item lists and their order), which the offset pass's result depends on.
Host code only: runs without a GPU."""
import ctypes as C

import numpy as np
import pytest


def _soup(seed, n, big_every=50):
    """Clusters of small triangles, a fraction of large ones (which stay in upper
    nodes), and a few degenerate ones."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-100, 100, (n, 1, 3)) * np.array([1.0, 1.0, 0.05])
    s = rng.uniform(0.05, 2.0, (n, 1, 1))
    s[::big_every] = 60.0
    tri = c + s * rng.uniform(-1, 1, (n, 3, 3))
    tri[7::97, 1] = tri[7::97, 0]          # degenerate: two equal vertices
    return np.ascontiguousarray(tri, dtype=np.float32).reshape(n, 9)


def _digest(lib, tri, threads):
    out = (C.c_uint64 * 3)()
    assert lib.ltrdbg_RefTreeDigest(tri.ctypes.data_as(C.c_void_p), tri.shape[0], threads, out)
    return tuple(out)


@pytest.mark.parametrize("seed,n", [(1, 3000), (2, 16000), (3, 60000), (4, 1025), (5, 5)])
def test_threaded_tree_equals_sequential(gpu, seed, n):
    tri = _soup(seed, n)
    seq = _digest(gpu, tri, 0)
    par = _digest(gpu, tri, 1)
    assert par == seq
    assert seq[0] >= 1 and seq[1] >= n    # every triangle is listed once (with its count words)


def test_empty_soup(gpu):
    tri = np.zeros((0, 9), np.float32)
    assert _digest(gpu, tri, 1) == _digest(gpu, tri, 0)
