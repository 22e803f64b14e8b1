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


def read_filterbank(path: str):
    """(header dict, float32[nchans][nsamples]) of a SIGPROC filterbank file
    (accel_read_filterbank): channel-major, channel c at fch1 + c * foff MHz."""
    info = N.FilterbankInfo()
    ptr = C.POINTER(C.c_float)()
    N.check(N.lib().accel_read_filterbank(str(path).encode(), C.byref(info), C.byref(ptr)))
    try:
        n = info.nchans * info.nsamples
        data = np.ctypeslib.as_array(ptr, shape=(n,)).copy().reshape(info.nchans, info.nsamples)
    finally:
        N.lib().accel_free_host(ptr)
    hdr = {f: getattr(info, f) for f, _ in info._fields_}
    hdr["source_name"] = info.source_name.decode(errors="replace")
    return hdr, data


def _main(argv=None) -> None:
    """Time one dedispersion of a seeded N(0,1) filterbank on cuda:0:
    python -m gpu_accelsearch_gb300.dedisperse --nchan 256 --nout 262144 --ndm 64"""
    import argparse
    import json

    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--nchan", type=int, default=1024)
    ap.add_argument("--nout", type=int, default=1 << 20)
    ap.add_argument("--ndm", type=int, default=256)
    ap.add_argument("--dm-step", type=float, default=1.0)
    ap.add_argument("--f-top", type=float, default=1500.0)
    ap.add_argument("--bandwidth", type=float, default=300.0)
    ap.add_argument("--tsamp", type=float, default=64e-6)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    dl, mx = dm_delays(a.nchan, a.f_top, -a.bandwidth / a.nchan, a.tsamp,
                       np.arange(a.ndm, dtype=np.float32) * a.dm_step)
    nsamp = a.nout + mx
    g = torch.Generator(device="cuda")
    g.manual_seed(31)
    fb = torch.randn((a.nchan, nsamp), generator=g, device="cuda", dtype=torch.float32)
    out = torch.empty((a.ndm, a.nout), device="cuda", dtype=torch.float32)
    st = torch.cuda.current_stream().cuda_stream
    dedisperse(fb.data_ptr(), a.nchan, nsamp, dl, out.data_ptr(), a.nout, st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(a.reps):
        dedisperse(fb.data_ptr(), a.nchan, nsamp, dl, out.data_ptr(), a.nout, st)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(a.reps, 1)
    print(json.dumps({"nchan": a.nchan, "nsamp": nsamp, "ndm": a.ndm, "nout": a.nout, "ms": ms,
                      "adds_per_s": a.ndm * a.nchan * a.nout / (ms / 1e3)}))


if __name__ == "__main__":
    _main()
