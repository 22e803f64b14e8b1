"""Dedispersion host side (no GPU): the library's delay table equals the
oracle's restatement of the dispersion delay, bad arguments are rejected,
and the oracle's direct sum undoes a known dispersion exactly."""
import ctypes as C

import numpy as np
import pytest

import __graft_entry__
from gpu_accelsearch_gb300 import native as N
from gpu_accelsearch_gb300.dedisperse import dm_delays
from oracle import oracle as O


@pytest.fixture(scope="module", autouse=True)
def lib():
    __graft_entry__.build_library()
    return N.lib()


@pytest.mark.parametrize("nchan,ftop,bw,tsamp", [(1024, 1510.0, -0.29296875, 64e-6),
                                                 (64, 1400.0, -4.6875, 64e-6),
                                                 (336, 1208.0, 0.5, 54.61333e-6),
                                                 (4096, 400.0, -0.048828125, 81.92e-6)])
def test_delays_match_oracle(nchan, ftop, bw, tsamp):
    dms = np.concatenate([np.arange(0, 100, 0.5), np.arange(100, 2000, 7.3)]).astype(np.float32)
    got, mx = dm_delays(nchan, ftop, bw, tsamp, dms)
    want = O.dm_delays(nchan, ftop, bw, tsamp, dms)
    assert np.array_equal(got, want)
    assert mx == int(want.max())
    assert (got[0] == 0).all() if dms[0] == 0 else True
    # delays grow with DM and towards the low end of the band
    assert (np.diff(got, axis=0) >= 0).all()
    lo_first = bw < 0
    assert (np.diff(got, axis=1) >= 0).all() if lo_first else (np.diff(got, axis=1) <= 0).all()


def test_bad_arguments_rejected(lib):
    d = (C.c_float * 2)(10.0, -1.0)
    out = (C.c_int * 8)()
    mx = C.c_int()
    assert lib.accel_dedisperse_delays(4, 1400.0, -1.0, 64e-6, d, 2, out, C.byref(mx)) == -1  # DM < 0
    assert lib.accel_dedisperse_delays(4, 1400.0, 0.0, 64e-6, d, 1, out, C.byref(mx)) == -1   # bw 0
    assert lib.accel_dedisperse_delays(4, 2.0, -1.0, 64e-6, d, 1, out, C.byref(mx)) == -1     # f <= 0
    # the device call checks its arguments before touching the GPU
    dl = (C.c_int * 4)(0, 1, 2, 3)
    fake = C.c_void_p(16)
    assert lib.accel_dedisperse(fake, 4, 100, dl, 1, fake, 98, None) == -1   # 98 + 3 > 100
    dl[0] = -1
    assert lib.accel_dedisperse(fake, 4, 100, dl, 1, fake, 10, None) == -1   # negative delay


def test_oracle_undoes_known_dispersion():
    rng = np.random.default_rng(3)
    nchan, nout = 16, 500
    x = rng.integers(-8, 8, nout).astype(np.float32)
    dl = O.dm_delays(nchan, 1400.0, -4.0, 64e-6, np.array([0.0, 25.0, 50.0], np.float32))
    mx = int(dl.max())
    fb = np.zeros((nchan, nout + mx), np.float32)
    for c in range(nchan):  # channel c sees the signal delay[1][c] samples later
        fb[c, dl[1, c]:dl[1, c] + nout] = x
    out = O.dedisperse(fb, dl, nout)
    assert np.array_equal(out[1], nchan * x)
    assert not np.array_equal(out[0], nchan * x)
