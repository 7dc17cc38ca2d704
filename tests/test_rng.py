"""Bulk AO random draws (ltrdbg_DrawRandFloats) against the C library's rand():
the values and the generator state afterwards must be those of n rand() calls."""
import ctypes as C

import numpy as np
import pytest

LIBC = C.CDLL(None)
LIBC.rand.restype = C.c_int
LIBC.srand.argtypes = [C.c_uint]
LIBC.initstate.restype = C.c_void_p
LIBC.initstate.argtypes = [C.c_uint, C.c_void_p, C.c_size_t]
LIBC.setstate.restype = C.c_void_p
LIBC.setstate.argtypes = [C.c_void_p]
RAND_MAX = np.float32(2147483647)


def _rand_floats(n):
    return np.array([np.float32(LIBC.rand()) / RAND_MAX for _ in range(n)], np.float32)


@pytest.fixture
def lib(built):
    from lighter_gb300 import library
    lib = library()
    lib.ltrdbg_DrawRandFloats.restype = None
    lib.ltrdbg_DrawRandFloats.argtypes = [C.c_void_p, C.c_uint32]
    return lib


def _draw(lib, n):
    out = np.zeros(max(n, 1), np.float32)
    lib.ltrdbg_DrawRandFloats(out.ctypes.data, n)
    return out[:n]


@pytest.mark.parametrize("seed", [1, 7, 123456789])
def test_bulk_draws_equal_rand_calls(lib, seed):
    sizes = [0, 1, 2, 30, 31, 32, 33, 1000, 4097]
    LIBC.srand(seed)
    want = [_rand_floats(n) for n in sizes]
    want_next = LIBC.rand()
    LIBC.srand(seed)
    got = [_draw(lib, n) for n in sizes]
    got_next = LIBC.rand()
    for n, w, g in zip(sizes, want, got):
        np.testing.assert_array_equal(g, w, err_msg=f"n={n}")
    assert got_next == want_next


def test_other_state_types_fall_back_to_rand(lib):
    buf = C.create_string_buffer(256)            # a type-4 state of the caller's
    old = LIBC.initstate(99, buf, 256)
    try:
        want = _rand_floats(500)
        LIBC.initstate(99, buf, 256)
        got = _draw(lib, 500)
        np.testing.assert_array_equal(got, want)
    finally:
        LIBC.setstate(old)
