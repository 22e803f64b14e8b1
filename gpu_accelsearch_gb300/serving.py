"""Python front end of the continuous-batching request server
(accel_server_* in include/accelsearch.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N
from .search import CAND_DTYPE


class Server:
    def __init__(self, hbm_budget_bytes=150e9, max_active=0, fftlen=8192, numharm=8, sigma=6.0,
                 chunk_segments=128, device=0, max_wait_s=1.0, max_chunk_segments=0):
        L = N.lib()
        cfg = N.ServerConfig()
        L.accel_server_config_init(C.byref(cfg))
        cfg.hbm_budget_bytes, cfg.max_active, cfg.fftlen = hbm_budget_bytes, max_active, fftlen
        cfg.numharm, cfg.sigma, cfg.chunk_segments, cfg.device = numharm, sigma, chunk_segments, device
        cfg.max_wait_s = max_wait_s
        cfg.max_chunk_segments = max_chunk_segments
        h = C.c_void_p()
        N.check(L.accel_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None):
            N.lib().accel_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, series: np.ndarray, dt: float, zmax: int) -> int:
        a = np.ascontiguousarray(series, dtype=np.float32)
        rid = C.c_longlong()
        N.check(N.lib().accel_server_submit(self._h, a.ctypes.data, a.size, dt, zmax, C.byref(rid)))
        self._keep[rid.value] = a  # the server reads it at admission
        return rid.value

    def wait(self, rid: int, timeout: float = -1.0) -> bool:
        done = C.c_int()
        N.check(N.lib().accel_server_wait(self._h, rid, timeout, C.byref(done)))
        return bool(done.value)

    def result(self, rid: int):
        """(candidates, latency in ms) of a finished request."""
        L = N.lib()
        n, lat = C.c_longlong(), C.c_double()
        N.check(L.accel_server_result(self._h, rid, None, 0, C.byref(n), C.byref(lat)))
        buf = (N.Candidate * max(n.value, 1))()
        N.check(L.accel_server_result(self._h, rid, buf, n.value, C.byref(n), C.byref(lat)))
        out = np.zeros(n.value, CAND_DTYPE)
        for i in range(n.value):
            c = buf[i]
            out[i] = (c.trial, c.step, c.r, c.z, c.numharm, c.power, c.sigma)
        return out, lat.value

    def timing(self, rid: int) -> dict:
        """Latency breakdown (ms) of a completed request: queue (submission to
        admission), prepare (admission's copy, transform and whitening
        launches), wait (prepared to its first launch group), search (first
        launch group to completion)."""
        out = (C.c_double * 4)()
        N.check(N.lib().accel_server_timing(self._h, rid, out))
        return dict(zip(("queue_ms", "prepare_ms", "wait_ms", "search_ms"), list(out)))

    def release(self, rid: int):
        N.check(N.lib().accel_server_release(self._h, rid))
        self._keep.pop(rid, None)

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(N.lib().accel_server_get_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}
