"""Python front end of the search: a thin, typed layer over the C ABI.

`AccelSearch` mirrors the reference pipeline (keithasr/gpu_accelsearch):

=============================  ==============================================
reference                      here
=============================  ==============================================
createSubharmonicInfo          AccelSearch(zmax, numharm, fftlen) (bank built
                               on the GPU at construction), .harmonics
realToComplexFFT               .rfft(series_dev, spec_dev)
deredden                       .whiten(spec_dev)
generate_harmonic_ffdot_data   .prepare_segments(wspec_dev, startr, out_dev)
 + perform_fft_harmonics
perform_convolution            .power_planes(dhalf_dev, nseg, planes_dev)
 + perform_inversefft
 + generate_fundamental_powers
perform_harmonic_summing       .sum_harmonics(planes_dev, startr, stage_dev)
 + search_ffdot_powers
main() step loop               .search(series, dt) / .search_spectra(...)
=============================  ==============================================

Device buffers are passed as integer device addresses (for example
``torch.Tensor.data_ptr()``); host inputs as numpy arrays.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native as N


@dataclass
class HarmonicInfo:
    harmnum: int
    maxharm: int
    zmax: int
    numzs: int
    fftlen: int
    halfwidth: int
    zlo: int
    plane_width: int


CAND_DTYPE = np.dtype([("trial", "i4"), ("step", "i4"), ("r", "f8"), ("z", "f8"),
                       ("numharm", "i4"), ("power", "f4"), ("sigma", "f4")])


def _native_dtype():
    """numpy view of N.Candidate (same offsets and size)."""
    return np.dtype({"names": ["trial", "step", "r", "z", "numharm", "power", "sigma"],
                     "formats": ["i4", "i4", "f8", "f8", "i4", "f4", "f4"],
                     "offsets": [N.Candidate.trial.offset, N.Candidate.step.offset,
                                 N.Candidate.r.offset, N.Candidate.z.offset,
                                 N.Candidate.numharm.offset, N.Candidate.power.offset,
                                 N.Candidate.sigma.offset],
                     "itemsize": C.sizeof(N.Candidate)})


def _to_native(cands: np.ndarray):
    buf = (N.Candidate * max(len(cands), 1))()
    if len(cands):
        view = np.frombuffer(buf, dtype=_native_dtype(), count=len(cands))
        for f in CAND_DTYPE.names:
            view[f] = cands[f]
    return buf


def _from_native(buf, n: int) -> np.ndarray:
    out = np.zeros(n, CAND_DTYPE)
    if n:
        view = np.frombuffer(buf, dtype=_native_dtype(), count=n)
        for f in CAND_DTYPE.names:
            out[f] = view[f]
    return out


def sift_candidates(cands: np.ndarray, min_dr: float = 15.0, maxharm: int = 8,
                    harm_dr: float = 1.0) -> np.ndarray:
    """accel_sift_candidates on a CAND_DTYPE array (see accelsearch.h)."""
    n = len(cands)
    src = _to_native(cands)
    dst = (N.Candidate * max(n, 1))()
    m = C.c_longlong()
    N.check(N.lib().accel_sift_candidates(src, n, float(min_dr), int(maxharm), float(harm_dr), dst,
                                          n, C.byref(m)))
    return _from_native(dst, m.value)


OPT_DTYPE = np.dtype([("trial", "i4"), ("step", "i4"), ("r", "f8"), ("z", "f8"), ("numharm", "i4"),
                      ("power", "f4"), ("sigma", "f4"), ("r_grid", "f8"), ("z_grid", "f8"),
                      ("harm_power", "f4", (16,)), ("f", "f8"), ("fdot", "f8"), ("period", "f8"),
                      ("pdot", "f8")])


def first_bin(nsamples: int, dt: float) -> int:
    return N.lib().accel_first_bin(nsamples, dt)


def autotune(zmax=200, numharm=8, fftlens=(4096, 8192, 16384), steps=64, template_fp16=False,
             device=0, short_transforms=None):
    """Pick the segment length and launch shape by timing them on this GPU.
    Returns (kwargs for AccelSearch, tuning dict, cells/s)."""
    L = N.lib()
    base = N.Config()
    L.accel_config_init(C.byref(base))
    base.zmax, base.numharm, base.template_fp16, base.device = zmax, numharm, int(template_fp16), device
    if short_transforms is not None:
        base.short_transforms = int(bool(short_transforms))
    fl = (C.c_int * len(fftlens))(*fftlens)
    best, tun, rate = N.Config(), N.Tuning(), C.c_double()
    N.check(L.accel_autotune(C.byref(base), fl, len(fftlens), steps, C.byref(best), C.byref(tun),
                             C.byref(rate)))
    kw = dict(zmax=zmax, numharm=numharm, fftlen=best.fftlen, template_fp16=template_fp16,
              chunk_segments=best.chunk_segments, device=device, short_transforms=bool(best.short_transforms))
    return kw, {"chunk_segments": tun.chunk_segments, "plane_split": tun.plane_split,
                "fused_sum": tun.fused_sum, "hsum_tile_rows": tun.hsum_tile_rows or 16}, rate.value


class AccelSearch:
    def __init__(self, zmax=200, numharm=8, fftlen=8192, uselen=0, sigma=6.0, numindep=1.0,
                 whiten_initbuf=6, whiten_maxbuf=200, template_fp16=False, chunk_segments=0,
                 cand_capacity=0, device=0, exact_rsqrt=False, short_transforms=None):
        L = N.lib()
        cfg = N.Config()
        L.accel_config_init(C.byref(cfg))
        cfg.zmax, cfg.numharm, cfg.fftlen, cfg.uselen = zmax, numharm, fftlen, uselen
        cfg.sigma, cfg.numindep = sigma, numindep
        cfg.whiten_initbuf, cfg.whiten_maxbuf = whiten_initbuf, whiten_maxbuf
        cfg.template_fp16 = int(bool(template_fp16))
        cfg.chunk_segments, cfg.cand_capacity, cfg.device = chunk_segments, cand_capacity, device
        cfg.exact_rsqrt = int(bool(exact_rsqrt))
        if short_transforms is not None:  # None: the library's default
            cfg.short_transforms = int(bool(short_transforms))
        self.config = cfg
        self.kwargs = dict(zmax=zmax, numharm=numharm, fftlen=fftlen, template_fp16=template_fp16,
                           chunk_segments=chunk_segments, device=device,
                           short_transforms=bool(cfg.short_transforms))
        h = C.c_void_p()
        N.check(L.accel_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.nh = L.accel_num_harmonics(h)
        self.nstages = L.accel_num_stages(h)
        self.uselen = L.accel_uselen(h)
        self.harmonics = []
        for i in range(self.nh):
            hi = N.Harmonic()
            N.check(L.accel_harmonic_info(h, i, C.byref(hi)))
            self.harmonics.append(HarmonicInfo(*[getattr(hi, f) for f, _ in hi._fields_]))
        ds, ps = C.c_longlong(), C.c_longlong()
        doff = (C.c_longlong * self.nh)()
        poff = (C.c_longlong * self.nh)()
        prow = (C.c_int * self.nh)()
        N.check(L.accel_layout(h, C.byref(ds), doff, C.byref(ps), poff, prow))
        self.dhalf_stride, self.plane_stride = ds.value, ps.value
        self.dhalf_off, self.plane_off = list(doff), list(poff)
        self.plane_row = list(prow)

    # ------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None):
            N.lib().accel_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------- queries
    def power_cuts(self):
        a = (C.c_float * self.nstages)()
        N.check(N.lib().accel_get_power_cuts(self._h, a))
        return np.array(a, np.float32)

    def set_power_cuts(self, cuts):
        a = (C.c_float * self.nstages)(*[float(x) for x in cuts])
        N.check(N.lib().accel_set_power_cuts(self._h, a))

    def step_count(self, nsamples: int, dt: float) -> int:
        return N.lib().accel_step_count(self._h, nsamples, dt)

    def bank_spectra(self, h: int):
        hi = self.harmonics[h]
        k = np.zeros((hi.numzs, hi.fftlen), np.complex64)
        f = np.zeros((hi.numzs, hi.fftlen), np.complex64)
        N.check(N.lib().accel_bank_spectra(self._h, h, k.ctypes.data, f.ctypes.data))
        return k, f

    def tuning(self) -> dict:
        t = N.Tuning()
        N.check(N.lib().accel_get_tuning(self._h, C.byref(t)))
        return {"chunk_segments": t.chunk_segments, "plane_split": t.plane_split,
                "fused_sum": t.fused_sum,
                "hsum_rowwise": t.hsum_rowwise, "serial_sum": t.serial_sum,
                "hsum_pipelined": t.hsum_pipelined, "graph": t.graph, "wait_test": t.wait_test,
                "persistent": t.persistent, "hsum_tile_rows": t.hsum_tile_rows,
                "hsum_row_copies": t.hsum_row_copies}

    def set_tuning(self, chunk_segments=None, plane_split=None, fused_sum=None,
                   hsum_rowwise=None, serial_sum=None, hsum_pipelined=None, graph=None,
                   wait_test=None, persistent=None, hsum_tile_rows=None, hsum_row_copies=None):
        cur = self.tuning()
        t = N.Tuning()
        t.chunk_segments = cur["chunk_segments"] if chunk_segments is None else chunk_segments
        t.plane_split = cur["plane_split"] if plane_split is None else int(plane_split)
        t.fused_sum = cur["fused_sum"] if fused_sum is None else int(fused_sum)
        t.hsum_rowwise = cur["hsum_rowwise"] if hsum_rowwise is None else int(hsum_rowwise)
        t.serial_sum = cur["serial_sum"] if serial_sum is None else int(serial_sum)
        t.hsum_pipelined = cur["hsum_pipelined"] if hsum_pipelined is None else int(hsum_pipelined)
        t.graph = cur["graph"] if graph is None else int(graph)
        t.wait_test = cur["wait_test"] if wait_test is None else int(wait_test)
        t.persistent = cur["persistent"] if persistent is None else int(persistent)
        t.hsum_tile_rows = cur["hsum_tile_rows"] if hsum_tile_rows is None else int(hsum_tile_rows)
        t.hsum_row_copies = cur["hsum_row_copies"] if hsum_row_copies is None else int(hsum_row_copies)
        N.check(N.lib().accel_set_tuning(self._h, C.byref(t)))

    def profile(self, enable: bool = True):
        N.check(N.lib().accel_profile(self._h, int(enable)))

    def stats(self) -> dict:
        st = N.Stats()
        N.check(N.lib().accel_get_stats(self._h, C.byref(st)))
        return {"launches": st.launches, "segments": st.segments, "cells": st.cells,
                "search_ms": st.search_ms, "searches": st.searches,
                "graph_launches": st.graph_launches, "graph_builds": st.graph_builds,
                "kinds": {k: {"launches": st.kind_launches[i], "ms": st.kind_ms[i]}
                          for i, k in enumerate(N.KINDS)}}

    def reset_stats(self):
        N.check(N.lib().accel_reset_stats(self._h))

    # -------------------------------------------------------------- stages
    def synchronize(self):
        N.check(N.lib().accel_synchronize(self._h))

    def rfft(self, series_dev: int, n: int, spec_dev: int):
        N.check(N.lib().accel_rfft(self._h, series_dev, n, spec_dev))

    def whiten(self, spec_dev: int, numbins: int):
        N.check(N.lib().accel_whiten(self._h, spec_dev, numbins))

    def prepare_segments(self, wspec_dev: int, numbins: int, startr, out_dev: int):
        s = np.ascontiguousarray(startr, dtype=np.int64)
        N.check(N.lib().accel_prepare_segments(self._h, wspec_dev, numbins,
                                               s.ctypes.data_as(C.POINTER(C.c_longlong)),
                                               s.size, out_dev))

    def power_planes(self, dhalf_dev: int, nseg: int, planes_dev: int):
        N.check(N.lib().accel_power_planes(self._h, dhalf_dev, nseg, planes_dev))

    def sum_harmonics(self, planes_dev: int, startr, stage_dev: int = 0) -> int:
        s = np.ascontiguousarray(startr, dtype=np.int64)
        n = C.c_longlong()
        N.check(N.lib().accel_sum_harmonics(self._h, planes_dev,
                                            s.ctypes.data_as(C.POINTER(C.c_longlong)), s.size,
                                            stage_dev or None, C.byref(n)))
        return n.value

    # -------------------------------------------------------------- search
    def search(self, series, dt, on_device=False, nsamples=None):
        """series: list of float32 numpy arrays (host) or device addresses."""
        n = len(series)
        ptrs = (C.c_void_p * n)()
        ns = (C.c_longlong * n)()
        dts = (C.c_double * n)()
        dtl = dt if isinstance(dt, (list, tuple, np.ndarray)) else [dt] * n
        keep = []
        for i, s in enumerate(series):
            if on_device:
                ptrs[i] = int(s)
                ns[i] = int(nsamples[i])
            else:
                a = np.ascontiguousarray(s, dtype=np.float32)
                keep.append(a)
                ptrs[i] = a.ctypes.data
                ns[i] = a.size
            dts[i] = float(dtl[i])
        nc = C.c_longlong()
        N.check(N.lib().accel_search(self._h, n, ptrs, ns, dts, int(bool(on_device)), C.byref(nc)))
        return nc.value

    def search_ptrs(self, ptrs, nsamples, dt, on_device: bool) -> int:
        """Search series given as raw addresses (device, or pinned host)."""
        n = len(ptrs)
        pa = (C.c_void_p * n)(*[int(p) for p in ptrs])
        ns = (C.c_longlong * n)(*[int(x) for x in nsamples])
        dtl = dt if isinstance(dt, (list, tuple, np.ndarray)) else [dt] * n
        dts = (C.c_double * n)(*[float(x) for x in dtl])
        nc = C.c_longlong()
        N.check(N.lib().accel_search(self._h, n, pa, ns, dts, int(bool(on_device)), C.byref(nc)))
        return nc.value

    def search_spectra(self, wspec_devs, numbins, rlo):
        n = len(wspec_devs)
        ptrs = (C.c_void_p * n)(*[int(p) for p in wspec_devs])
        nb = (C.c_longlong * n)(*[int(x) for x in numbins])
        rl = (C.c_longlong * n)(*[int(x) for x in rlo])
        nc = C.c_longlong()
        N.check(N.lib().accel_search_spectra(self._h, n, ptrs, nb, rl, C.byref(nc)))
        return nc.value

    def trial_spectrum(self, trial: int):
        """(device address, numbins) of trial's whitened spectrum from the last search."""
        p = C.c_void_p()
        nb = C.c_longlong()
        N.check(N.lib().accel_trial_spectrum(self._h, int(trial), C.byref(p), C.byref(nb)))
        return p.value, nb.value

    def optimize(self, cands: np.ndarray, rlo, tobs, spectra=None, refine: bool = True) -> np.ndarray:
        """accel_optimize_candidates.  spectra: [(device address, numbins)] per
        trial (default: the whitened spectra of the last search); rlo and
        tobs: the first bin searched and the observation time (s) of every
        trial (or one value for all)."""
        n = len(cands)
        if spectra is None:
            nt = int(cands["trial"].max()) + 1 if n else 1
            spectra = [self.trial_spectrum(t) for t in range(nt)]
        nt = len(spectra)
        per = lambda v: list(v) if isinstance(v, (list, tuple, np.ndarray)) else [v] * nt
        ptrs = (C.c_void_p * nt)(*[int(p) for p, _ in spectra])
        nbs = (C.c_longlong * nt)(*[int(b) for _, b in spectra])
        rl = (C.c_longlong * nt)(*[int(x) for x in per(rlo)])
        tob = (C.c_double * nt)(*[float(x) for x in per(tobs)])
        src = _to_native(cands)
        dst = (N.Optimized * max(n, 1))()
        N.check(N.lib().accel_optimize_candidates(self._h, nt, ptrs, nbs, rl, tob, src, n, int(refine),
                                                  dst))
        out = np.zeros(n, OPT_DTYPE)
        for k in range(n):
            o = dst[k]
            c = o.cand
            out[k] = (c.trial, c.step, c.r, c.z, c.numharm, c.power, c.sigma, o.r_grid, o.z_grid,
                      tuple(o.harm_power), o.f, o.fdot, o.period, o.pdot)
        return out

    def candidates(self) -> np.ndarray:
        L = N.lib()
        n = C.c_longlong()
        N.check(L.accel_candidates(self._h, None, 0, C.byref(n)))
        buf = (N.Candidate * max(n.value, 1))()
        N.check(L.accel_candidates(self._h, buf, n.value, C.byref(n)))
        out = np.zeros(n.value, CAND_DTYPE)
        raw = np.frombuffer(buf, dtype=np.uint8, count=n.value * C.sizeof(N.Candidate))
        if n.value:
            view = np.ndarray(n.value, dtype=np.dtype({
                "names": ["trial", "step", "r", "z", "numharm", "power", "sigma"],
                "formats": ["i4", "i4", "f8", "f8", "i4", "f4", "f4"],
                "offsets": [N.Candidate.trial.offset, N.Candidate.step.offset,
                            N.Candidate.r.offset, N.Candidate.z.offset,
                            N.Candidate.numharm.offset, N.Candidate.power.offset,
                            N.Candidate.sigma.offset],
                "itemsize": C.sizeof(N.Candidate)}), buffer=raw)
            for f in CAND_DTYPE.names:
                out[f] = view[f]
        return out
