"""Whitening block plan (deredden's recurrence, bpd_noise.c:33-79) on the
host, through the C ABI: equal to a restatement of the reference's loop,
free of overflow up to the largest accepted spectrum (2^31 - 1 bins, block
starts and lengths are int as in the reference), and refusals beyond it."""
import ctypes as C
import math

import numpy as np
import pytest

import __graft_entry__
from gpu_accelsearch_gb300 import native as N

INT_MAX = (1 << 31) - 1


@pytest.fixture(scope="module")
def lib():
    __graft_entry__.build_library()
    return N.lib()


def ref_blocks(numbins, init, maxb):
    # the reference's loop: binnum and buflen are int, the width is
    # (int)(initialbuflen * log(binnum)) capped at maxbuflen
    out = [(1, init)]
    binnum, buflen = 1 + init, min(int(init * math.log(1 + init)), maxb)
    while binnum + buflen < numbins:
        out.append((binnum, buflen))
        binnum += buflen
        buflen = min(int(init * math.log(binnum)), maxb)
    return out


def plan(lib, numbins, init, maxb, cap=None):
    n = C.c_longlong()
    rc = lib.accel_whiten_blocks(numbins, init, maxb, None, None, 0, C.byref(n))
    if rc:
        return rc, None
    cap = n.value if cap is None else cap
    s = (C.c_int * max(cap, 1))()
    ln = (C.c_int * max(cap, 1))()
    assert lib.accel_whiten_blocks(numbins, init, maxb, s, ln, cap, C.byref(n)) == 0
    return 0, (n.value, list(zip(s[:min(cap, n.value)], ln[:min(cap, n.value)])))


@pytest.mark.parametrize("numbins,init,maxb", [(8, 6, 200), (1 << 17, 6, 200), (12345, 6, 200),
                                               (1 << 17, 1000, 1000), (1 << 20, 600, 4096),
                                               (1 << 16, 3, 2000), (3 << 20, 6, 200)])
def test_plan_equals_reference_loop(lib, numbins, init, maxb):
    rc, (n, blocks) = plan(lib, numbins, init, maxb)
    assert rc == 0
    assert blocks == ref_blocks(numbins, init, maxb) and n == len(blocks)


def test_largest_spectrum_without_overflow(lib):
    # 2^31 - 1 bins: every block start + length stays below numbins, starts
    # increase, and the wide-block plan equals the reference loop evaluated
    # in unbounded integers
    for init, maxb in ((3000, 49152), (1000, 1000)):
        rc, (n, blocks) = plan(lib, INT_MAX, init, maxb)
        assert rc == 0
        assert blocks == ref_blocks(INT_MAX, init, maxb)
        st = np.array([b[0] for b in blocks], np.int64)
        ln = np.array([b[1] for b in blocks], np.int64)
        assert (np.diff(st) == ln[:-1]).all() and (st + ln < INT_MAX).all() and (ln >= 1).all()
    # default widths (6 ln(binnum), at most 128 bins below 2^31): about
    # 1.76e7 blocks, counted without storing them
    n = C.c_longlong()
    assert lib.accel_whiten_blocks(INT_MAX, 6, 200, None, None, 0, C.byref(n)) == 0
    assert 1.7e7 < n.value < 1.8e7


@pytest.mark.parametrize("numbins,init,maxb", [(1 << 31, 6, 200), (1 << 32, 3000, 49152), (7, 6, 200),
                                               (1 << 20, 0, 200), (1 << 20, 6, 0)])
def test_out_of_range_refused(lib, numbins, init, maxb):
    n = C.c_longlong()
    assert lib.accel_whiten_blocks(numbins, init, maxb, None, None, 0, C.byref(n)) == -1


def test_noalloc_refuses_beyond_int_range_before_the_device(lib):
    # checked on the host before any CUDA call, so this runs without a GPU
    buf = (C.c_float * 4)()
    rc = lib.accel_whiten_noalloc(C.cast(buf, C.c_void_p), 1 << 31, 3000, 49152, None)
    assert rc == -1
    assert "out of range" in lib.accel_last_error().decode()
