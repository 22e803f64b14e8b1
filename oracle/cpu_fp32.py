"""FP32 CPU restatement of the reference search (test infrastructure and the
CPU baseline only: bench.py's cpu_baseline leg and --impl reference time it,
tests check it; the product library never imports it).

It follows the reference pipeline's arithmetic and layout step by step,
the way bpd_search.cu runs it on the GPU, with the FFTs in single precision
(scipy.fft, pocketfft) instead of cuFFT:
  * segment data -- the reference's host preparation (bpd_search.cu:130-184),
    taken from the oracle's bit-exact C restatement (segment_data);
  * forward FFT of each harmonic's spread segment (bpd_search.cu:228-240);
  * multiply by the conjugate template spectrum (convolveSignal,
    bpd_gpu_kernels.cu:39-81);
  * unnormalised inverse FFT of every row (bpd_search.cu:276-287);
  * |y|^2 / L^2 from column 2 hw0 (generatePowers, bpd_gpu_kernels.cu:84-116);
  * harmonic sums with the reference's index arithmetic -- rind =
    (ushort)((subr - rlo_h) 2), subr = (int)(2 rr f + 0.5) / 2, subz = (int)(zz f)
    truncated, zind = (int)((subz - zlo_h) / 2) (addPowers,
    bpd_gpu_kernels.cu:119-170) -- stages after 1, 2, 4, 8 harmonics
    (bpd_search.cu:350), and the candidate cut the reference leaves as a stub.
Steps are spread over a process pool (spawn: safe after CUDA has been
initialised in the parent), one step at a time per process.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time

import numpy as np

from oracle import oracle as O


class Fp32Search:
    def __init__(self, zmax: int, numharm: int, uselen: int):
        import scipy.fft as sfft
        self.sfft = sfft
        self.zmax, self.numharm, self.uselen = zmax, numharm, uselen
        self.geom = O.bank_geometry(zmax, numharm, uselen)  # harmnum, maxharm, zmax_h, numzs, L, hw0, zlo
        self.nh = len(self.geom)
        self.tconj = []
        for p, q, zmax_h, numzs, L, hw0, zlo in self.geom:
            t = np.stack([O.wrapped_template(int(L), int(-zmax_h + 2 * j)) for j in range(int(numzs))])
            self.tconj.append(np.conj(sfft.fft(t, axis=1, workers=1)).astype(np.complex64))
        self.numzs0 = int(self.geom[0, 3])
        self.zlo0 = int(self.geom[0, 6])

    def harmonic_powers(self, w, startr: int, h: int):
        """The f-dot plane of harmonic h from column 2 hw0 on: |y|^2 / L^2."""
        p, q, zmax_h, numzs, L, hw0, zlo = (int(v) for v in self.geom[h])
        U = self.uselen
        rlo, rhi, _, _ = O.step_ffdot(p, q, self.zmax, U, float(startr), startr + U // 2 - 0.5)
        seg = O.segment_data(w, rlo, rhi, hw0, L)
        d = self.sfft.fft(seg, workers=1)
        y = self.sfft.ifft(self.tconj[h] * d[None, :], axis=1, norm="forward", workers=1)
        y = y[:, 2 * hw0:]
        pw = (y.real * y.real + y.imag * y.imag).astype(np.float32)
        pw *= np.float32(1.0 / (L * L))
        return pw, rlo, zlo

    def step(self, w, startr: int):
        """Stage sums (nstages, numzs0, uselen) of one overlap-save step."""
        U = self.uselen
        p0, _, _ = self.harmonic_powers(w, startr, 0)
        s = p0[:, :U].copy()
        stages = [s.copy()]
        i = np.arange(U, dtype=np.float64)
        zz = (self.zlo0 + 2 * np.arange(self.numzs0)).astype(np.float64)
        for h in range(1, self.nh):
            pw, rlo_h, zlo_h = self.harmonic_powers(w, startr, h)
            f = float(self.geom[h, 0]) / float(self.geom[h, 1])
            rr = startr + i * 0.5
            subr = np.floor(2.0 * rr * f + 0.5) * 0.5
            rind = ((subr - rlo_h) * 2.0).astype(np.int64) & 0xFFFF
            subz = np.trunc(zz * f)
            zind = np.trunc((subz - zlo_h) * 0.5).astype(np.int64)
            s += pw[zind[:, None], rind[None, :]]
            if ((h + 1) & h) == 0:
                stages.append(s.copy())
        return np.stack(stages)


_W = {}


def _init(zmax, numharm, uselen, wspec):
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    _W["s"] = Fp32Search(zmax, numharm, uselen)
    _W["w"] = wspec


def _run_steps(args):
    startrs, cuts = args
    s, w = _W["s"], _W["w"]
    ncand = 0
    for sr in startrs:
        st = s.step(w, int(sr))
        for k in range(st.shape[0]):
            ncand += int(np.count_nonzero(st[k] > cuts[k]))
    return ncand


class StepPool:
    """A spawn process pool holding one Fp32Search and the whitened spectrum
    per process; run() searches steps one per task and times them (pool
    start-up and the template spectra stay outside the timing)."""

    def __init__(self, zmax, numharm, uselen, wspec, processes=None):
        self.processes = processes or os.cpu_count() or 1
        ctx = mp.get_context("spawn")
        self.pool = ctx.Pool(self.processes, initializer=_init, initargs=(zmax, numharm, uselen, wspec))

    def run(self, startrs, cuts):
        """(seconds, candidates) for the given step start bins."""
        self.pool.map(_run_steps, [([startrs[0]], cuts)] * self.processes)  # every worker warm
        t = time.perf_counter()
        nc = sum(self.pool.map(_run_steps, [([sr], cuts) for sr in startrs], chunksize=1))
        return time.perf_counter() - t, nc

    def close(self):
        self.pool.close()
        self.pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def timed_search(zmax, numharm, uselen, wspec, startrs, cuts, processes=None):
    """Search the given steps with a fresh pool; returns (seconds, candidates,
    processes)."""
    with StepPool(zmax, numharm, uselen, wspec, processes) as p:
        el, nc = p.run(startrs, cuts)
    return el, nc, p.processes
