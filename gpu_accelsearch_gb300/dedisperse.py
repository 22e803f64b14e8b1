"""Incoherent dedispersion of a filterbank into DM-trial series on the GPU
(accel_dedisperse_delays / accel_dedisperse in include/accelsearch.h): the
step that produces the time series the search takes."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N


def dm_delays(nchan: int, f_top_mhz: float, chan_bw_mhz: float, tsamp: float, dms) -> tuple:
    """Per (DM trial, channel) delays in samples, int32[ndm][nchan], and the
    largest of them."""
    d = np.ascontiguousarray(dms, dtype=np.float32)
    out = np.zeros((d.size, nchan), np.int32)
    mx = C.c_int()
    N.check(N.lib().accel_dedisperse_delays(nchan, f_top_mhz, chan_bw_mhz, tsamp,
                                            d.ctypes.data_as(C.POINTER(C.c_float)), d.size,
                                            out.ctypes.data_as(C.POINTER(C.c_int)), C.byref(mx)))
    return out, mx.value


def dedisperse(filterbank_dev: int, nchan: int, nsamp: int, delays: np.ndarray, out_dev: int,
               nout: int, stream: int = 0) -> None:
    """out_dev[d][t] (float32[ndm][nout], device) = sum over channels of the
    device filterbank float32[nchan][nsamp] shifted by delays[d][c]."""
    dl = np.ascontiguousarray(delays, dtype=np.int32)
    if dl.ndim != 2 or dl.shape[1] != nchan:
        raise ValueError("delays must be int32[ndm][nchan]")
    N.check(N.lib().accel_dedisperse(filterbank_dev, nchan, nsamp,
                                     dl.ctypes.data_as(C.POINTER(C.c_int)), dl.shape[0], out_dev,
                                     nout, stream or None))
