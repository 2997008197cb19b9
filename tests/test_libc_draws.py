"""The drop-in's draws of the process's libc rand() sequence
(moc_ref_libc_draws, moc_libc_rand.cpp): the same values as rand() calls, and
libc's state left where those calls leave it, for glibc's default state, its
other additive states, and the type-0 state that falls back to rand() itself.
The serial reference draws one rand() per sub-segment (src/solver.c:476-483).
No GPU: the draws are host code."""
import ctypes as C
import platform

import numpy as np
import pytest

libc = C.CDLL(None)
libc.rand.restype = C.c_int
libc.srand.argtypes = [C.c_uint]
libc.initstate.argtypes = [C.c_uint, C.c_char_p, C.c_size_t]
libc.initstate.restype = C.c_void_p
libc.setstate.argtypes = [C.c_void_p]
libc.setstate.restype = C.c_void_p

glibc = platform.libc_ver()[0] == "glibc"


def _draws(n):
    from simplemoc_gb300 import refabi
    out = np.zeros(max(n, 1), dtype=np.int32)
    bulk = C.c_int(-1)
    rc = refabi.lib().moc_ref_libc_draws(out.ctypes.data_as(C.POINTER(C.c_int32)), n,
                                         C.byref(bulk))
    assert rc == 0
    return out[:n], bulk.value


def _calls(n):
    return np.array([libc.rand() for _ in range(n)], dtype=np.int32)


@pytest.mark.parametrize("n", [0, 1, 30, 31, 1000, 70001])
def test_default_state_matches_rand_calls(n):
    libc.srand(20260104)
    want = _calls(n)
    after = libc.rand()
    libc.srand(20260104)
    got, bulk = _draws(n)
    assert np.array_equal(got, want)
    assert libc.rand() == after            # libc continues where n calls leave it
    if glibc and n:
        assert bulk == 1


def test_threaded_draws_match_rand_calls():
    """Past 2^22 values the draws are split over host threads, each starting
    from a window computed by polynomial jump-ahead."""
    n = (1 << 22) + 12345
    libc.srand(99)
    for _ in range(17):
        libc.rand()
    want = _calls(n)
    after = [libc.rand() for _ in range(40)]
    libc.srand(99)
    for _ in range(17):
        libc.rand()
    got, _ = _draws(n)
    assert np.array_equal(got, want)
    assert [libc.rand() for _ in range(40)] == after


@pytest.mark.parametrize("size,kind", [(32, "type 1"), (64, "type 2"), (128, "type 3"),
                                       (256, "type 4"), (16, "type 0")])
def test_other_generator_states(size, kind):
    buf = C.create_string_buffer(size)
    old = libc.initstate(7, buf, size)
    try:
        for _ in range(3):
            libc.rand()
        snap = buf.raw
        want = _calls(5000)
        after = libc.rand()
        # the same state again: restore the buffer and its position
        C.memmove(buf, snap, size)
        libc.setstate(buf)
        libc.initstate(7, buf, size)
        for _ in range(3):
            libc.rand()
        got, bulk = _draws(5000)
        assert np.array_equal(got, want), kind
        assert libc.rand() == after, kind
        if glibc:
            assert bulk == (0 if kind == "type 0" else 1), kind
    finally:
        libc.setstate(old)


def test_rejects_bad_arguments():
    from simplemoc_gb300 import refabi
    lb = refabi.lib()
    assert lb.moc_ref_libc_draws(None, 5, None) == 1
    assert lb.moc_ref_libc_draws(None, -1, None) == 1
    assert lb.moc_ref_libc_draws(None, 0, None) == 0
