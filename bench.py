#!/usr/bin/env python
"""f-fdot cells/s of the Fourier-domain acceleration search on one GB300.

One "step" = one whole batched search over a fixed synthetic batch of DM
trials (the batched configuration: trial lengths uniform in
{2^20, 2^21, 2^22, 3*2^20} samples at dt = 64 us, 10% with one injected
accelerated sinusoid, zmax = 200, 8 harmonics, 8192-point segments):
R2C FFT, whitening, every overlap-save step of every trial (segment
preparation, fused correlation / inverse FFT / power plane, harmonic sum
and threshold) and the read-back of the candidate list.

    value   cells/s with the series already in HBM when timing starts
    e2e     the same through the C ABI from pinned host buffers (host->device
            copy of every series and device->host read of the candidates
            inside the timed region)

A cell is one fundamental f-fdot point (r step 1/2, z step 2) carried
through all harmonic stages.  --impl reference times the CPU oracle (a
restatement of the reference pipeline, FP64) on a bounded sample instead.
Under torchrun every rank searches its own trials (no collective); rank 0
prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LENGTHS = [1 << 20, 1 << 21, 1 << 22, 3 << 20]
DT = 64e-6
ZMAX, NUMHARM, FFTLEN = 200, 8, 8192
METRIC = "f-fdot cells/s (zmax=200, 8 harmonics, batched)"
# algorithmic HBM bytes per fundamental cell at zmax=200 / 8 harmonics:
# every harmonic plane written once (4 B) and read once (4 B) per cell of
# that plane; the planes hold 3.205x the fundamental cells.
PLANE_RATIO = None  # computed from the bank geometry


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--trials", type=int, default=256, help="DM trials per GPU")
    ap.add_argument("--chunk", type=int, default=0, help="segments per launch group (0: auto)")
    ap.add_argument("--fftlen", type=int, default=0,
                    help="segment length; 0: chosen by the autotuner among 4096/8192/16384")
    ap.add_argument("--split", type=int, default=-1, help="plane kernel layout (-1: autotuner)")
    ap.add_argument("--tuning", default="", help="JSON of extra accel_tuning fields to apply")
    ap.add_argument("--short-transforms", type=int, default=-1, choices=[-1, 0, 1],
                    help="1: short (R*2^k) segment transforms, 0: the reference's powers of two, "
                         "-1: the library default")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--precision-seeds", type=int, default=100,
                    help="seeds of the FP16-template precision report (0: skip)")
    ap.add_argument("--serving-seconds", type=float, default=5.0,
                    help="duration of the Poisson arrival process of the serving leg (0: skip)")
    ap.add_argument("--serving-chunk", type=int, default=128, help="segments per launch group of the server")
    ap.add_argument("--serving-max-chunk", type=int, default=0,
                    help="largest launch group of the server, sized by the backlog (0: fixed groups)")
    ap.add_argument("--serving-lengths", default="log-uniform", choices=["log-uniform", "octaves"],
                    help="request lengths: log-uniform 2^18..2^23 (every request a new length), or "
                         "rounded down to powers of two")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


# ------------------------------------------------------------------ clocks
class Clocks:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def start(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 8:
                    rows.append(p)
        os.unlink(self.f.name)
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- workload
def make_batch(ntrials: int, seed: int):
    """Seeded trial lengths and signals (host description)."""
    rng = np.random.default_rng(seed)
    lengths = [int(x) for x in rng.choice(LENGTHS, ntrials)]
    sigs = []
    for n in lengths:
        if rng.random() < 0.10:
            sigs.append((float(rng.uniform(0.02, 0.1)), float(rng.uniform(1e4, min(1e6, 0.4 * n))),
                         float(rng.uniform(-150, 150))))
        else:
            sigs.append(None)
    return lengths, sigs


def device_series(torch, lengths, sigs, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    out = []
    for n, s in zip(lengths, sigs):
        x = torch.randn(n, generator=g, device="cuda", dtype=torch.float32)
        if s is not None:
            amp, r0, z = s
            t = torch.arange(n, device="cuda", dtype=torch.float64) / n
            x += (amp * torch.cos(2 * np.pi * (r0 * t + 0.5 * z * t * t))).float()
        out.append(x)
    return out


# ----------------------------------------------------------------- serving
def smooth_length(n: int) -> int:
    """Smallest even 7-smooth length >= n (observations are padded to
    FFT-friendly lengths)."""
    m = n + (n & 1)
    while True:
        k = m
        for p in (2, 3, 5, 7):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 2

def run_serving(seconds: float, device: int, rate: float = 200.0, chunk: int = 128, lengths: str = "log-uniform",
                max_chunk: int = 0):
    """The serving configuration: Poisson arrivals at `rate` per second of
    DM-trial series with lengths log-uniform in 2^18..2^23 samples, zmax
    uniform in {50, 100, 200, 300}, 5% with an injected signal, admitted
    against a 150 GB HBM budget.  Requests are slices of a pool of seeded
    host series (the server reads a request's samples when it admits it)."""
    from gpu_accelsearch_gb300.serving import Server
    from gpu_accelsearch_gb300.synth import synth_series
    rng = np.random.default_rng(4242)
    nmax = 1 << 23
    pool = [synth_series(nmax, seed=700 + i) for i in range(8)]
    sig = [synth_series(nmax, seed=800 + i, signals=[(0.05, 1e5 * (i + 1), 20.0 * (i - 2))])
           for i in range(4)]
    t, arrivals = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        n = smooth_length(int(2 ** rng.uniform(18, 23)))
        if lengths == "octaves":  # a few fixed lengths: one R2C plan each
            n = 1 << int(np.floor(np.log2(n)))
        zmax = int(rng.choice([50, 100, 200, 300]))
        src = sig[rng.integers(len(sig))] if rng.random() < 0.05 else pool[rng.integers(len(pool))]
        arrivals.append((t, src[:n], zmax))
    srv = Server(hbm_budget_bytes=150e9, fftlen=8192, numharm=8, chunk_segments=chunk, device=device,
                 max_chunk_segments=max_chunk)
    for z in (50, 100, 200, 300):  # build the four banks outside the measurement
        srv.wait(srv.submit(pool[0][: 1 << 18], DT, z), -1)
    base = srv.stats()
    t0 = time.perf_counter()
    ids = []
    for ta, x, z in arrivals:
        dly = t0 + ta - time.perf_counter()
        if dly > 0:
            time.sleep(dly)
        ids.append(srv.submit(x, DT, z))
    lats, parts = [], []
    for rid in ids:
        srv.wait(rid, -1)
        lats.append(srv.result(rid)[1])
    wall = time.perf_counter() - t0
    for rid in ids:
        parts.append(srv.timing(rid))
    # latency by length class (octaves of the sample count), with the median
    # of each part of it
    by_class = {}
    for (ta, x, z), lat, pt in zip(arrivals, lats, parts):
        k = int(np.floor(np.log2(x.size)))
        by_class.setdefault(k, []).append((lat, pt))
    classes = {}
    for k, v in sorted(by_class.items()):
        lv = [a for a, _ in v]
        classes[f"2^{k}..2^{k + 1}"] = dict(
            {"requests": len(v), "p50_ms": float(np.percentile(lv, 50)), "p99_ms": float(np.percentile(lv, 99))},
            **{"median_" + key: float(np.median([p[key] for _, p in v]))
               for key in ("queue_ms", "prepare_ms", "wait_ms", "search_ms")})
    st = srv.stats()
    srv.close()
    cells = st["cells"] - base["cells"]
    gpu_s = (st["gpu_ms"] - base["gpu_ms"]) / 1e3
    lats = np.array(lats)
    return {"requests": len(ids), "offered_rate_per_s": rate, "arrival_seconds": seconds,
            "p50_ms": float(np.percentile(lats, 50)), "p99_ms": float(np.percentile(lats, 99)),
            "mean_ms": float(lats.mean()), "max_ms": float(lats.max()),
            "cells_per_s": cells / wall, "cells_per_gpu_s": cells / gpu_s if gpu_s else None,
            "admission_thread_s": (st["admit_ms"] - base["admit_ms"]) / 1e3,
            "scheduler_group_s": (st["group_ms"] - base["group_ms"]) / 1e3,
            "gpu_search_s": gpu_s,
            "gpu_gap_s": (st["gap_ms"] - base["gap_ms"]) / 1e3,
            "gpu_idle_s": (st["idle_ms"] - base["idle_ms"]) / 1e3,
            "scheduler_wait_s": (st["wait_ms"] - base["wait_ms"]) / 1e3,
            "scheduler_launch_s": (st["launch_ms"] - base["launch_ms"]) / 1e3,
            "gpu_prepare_s": (st["prep_gpu_ms"] - base["prep_gpu_ms"]) / 1e3,
            "groups": st["groups"] - base["groups"],
            "segments_per_group": (st["group_segments"] - base["group_segments"]) / max(1, st["groups"] - base["groups"]),
            "wall_s": wall, "hbm_budget_bytes": 150e9, "max_wait_s": 1.0, "chunk_segments": chunk,
            "max_chunk_segments": max_chunk,
            "lengths": lengths,
            "by_length": classes,
            "workload": "Poisson arrivals, lengths log-uniform 2^18..2^23 (rounded up to even "
                        "7-smooth lengths), "
                        "zmax uniform in {50,100,200,300}, 5% with a signal, L=8192, 8 harmonics, "
                        "continuous batching (accel_server)"}


# ------------------------------------------------------------- dedispersion
def run_dedisperse(device: int, reps: int = 3):
    """Incoherent dedispersion upstream of the search: a 1024-channel
    filterbank (1500 MHz top, 300 MHz band, 64 us samples, N(0,1) float32)
    into 256 DM trials 0..255 pc cm^-3 of 2^20 samples each, timed with
    CUDA events after a warm-up (inputs larger than L2)."""
    import torch
    from gpu_accelsearch_gb300.dedisperse import dedisperse, dm_delays
    nchan, nout, ndm = 1024, 1 << 20, 256
    dl, mx = dm_delays(nchan, 1500.0, -300.0 / nchan, DT, np.arange(ndm, dtype=np.float32))
    nsamp = nout + mx
    g = torch.Generator(device="cuda")
    g.manual_seed(31)
    fb = torch.randn((nchan, nsamp), generator=g, device="cuda", dtype=torch.float32)
    out = torch.empty((ndm, nout), device="cuda", dtype=torch.float32)
    st = torch.cuda.current_stream().cuda_stream
    dedisperse(fb.data_ptr(), nchan, nsamp, dl, out.data_ptr(), nout, st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        dedisperse(fb.data_ptr(), nchan, nsamp, dl, out.data_ptr(), nout, st)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / reps
    adds = float(ndm) * nchan * nout
    byts = 4.0 * (nchan * nsamp + ndm * nout)
    del fb, out
    return {"workload": "1024 channels x (2^20 + %d) samples -> 256 DM trials x 2^20 samples" % mx,
            "ms": sec * 1e3, "dm_samples_per_s": ndm * nout / sec, "adds_per_s": adds / sec,
            "algorithmic_GBs": byts / sec / 1e9,
            "note": "algorithmic bytes: the filterbank read once and the trials written once"}


# --------------------------------------------------------------- precision
def precision_report(seeds: int, device: int):
    """FP16 folded templates (scaled per template) against FP32 templates
    and the FP64 oracle on the single-trial configuration: N = 2^22, three
    injected signals per seed (r in [1e4, 1e6], z in [-150, 150], amplitude
    in [0.02, 0.1]), zmax = 200, 8 harmonics, L = 8192, sigma = 6."""
    import torch
    from gpu_accelsearch_gb300.search import AccelSearch
    from oracle import oracle as O
    n = 1 << 22
    s32 = AccelSearch(zmax=ZMAX, numharm=NUMHARM, fftlen=FFTLEN, device=device)
    s16 = AccelSearch(zmax=ZMAX, numharm=NUMHARM, fftlen=FFTLEN, template_fp16=True, device=device)
    U, half = s32.uselen, s32.uselen // 2
    rec16 = rec32 = inj = 0
    agree = tot32 = 0
    worst_err, err_sum, err_cells = 0.0, 0.0, 0
    orc = None
    for seed in range(seeds):
        rng = np.random.default_rng(9000 + seed)
        sigs = [(float(rng.uniform(0.02, 0.1)), float(rng.uniform(1e4, 1e6)), float(rng.uniform(-150, 150)))
                for _ in range(3)]
        x = device_series(torch, [n], [None], seed=5000 + seed)[0]
        t = torch.arange(n, device="cuda", dtype=torch.float64) / n
        for amp, r0, z in sigs:
            x += (amp * torch.cos(2 * np.pi * (r0 * t + 0.5 * z * t * t))).float()
        torch.cuda.synchronize()
        res = []
        for s in (s32, s16):
            s.search([x.data_ptr()], DT, on_device=True, nsamples=[n])
            res.append(s.candidates())
        c32, c16 = res
        k32 = {(int(c["step"]), float(c["r"]), float(c["z"]), int(c["numharm"])) for c in c32}
        k16 = {(int(c["step"]), float(c["r"]), float(c["z"]), int(c["numharm"])) for c in c16}
        agree += len(k32 & k16)
        tot32 += len(k32)
        for amp, r0, z in sigs:
            inj += 1
            for c, cnt in ((c32, 0), (c16, 1)):
                hit = np.any((np.abs(c["r"] - (r0 + z / 2)) <= 2.0) & (np.abs(c["z"] - z) <= 4.0))
                if cnt == 0:
                    rec32 += int(hit)
                else:
                    rec16 += int(hit)
        # power error against the FP64 oracle on the step holding the first signal
        if orc is None:
            orc = O.Oracle(ZMAX, NUMHARM, U)
            from concurrent.futures import ThreadPoolExecutor
            pool = ThreadPoolExecutor(max_workers=len(s16.harmonics))
        spec = torch.fft.rfft(x.double()).to(torch.complex64)[: n // 2].cpu().numpy()
        w = O.deredden(spec)
        rlo = int(np.floor(np.float32(n) * np.float32(DT)))
        step = max(0, int((sigs[0][1] + sigs[0][2] / 2 - rlo) // half))
        startr = rlo + step * half
        d = torch.from_numpy(w.view(np.float32).copy()).cuda()
        dh = torch.zeros(s16.dhalf_stride * 2, dtype=torch.float32, device="cuda")
        pl = torch.zeros(s16.plane_stride, dtype=torch.float32, device="cuda")
        s16.prepare_segments(d.data_ptr(), w.size, [startr], dh.data_ptr())
        s16.power_planes(dh.data_ptr(), 1, pl.data_ptr())
        P = pl.cpu().numpy()
        # the oracle's planes of the eight harmonics in parallel (the C
        # calls release the interpreter lock)
        p64s = list(pool.map(lambda h: orc.harmonic_plane(w, float(startr), h),
                             range(len(s16.harmonics))))
        for h, hi in enumerate(s16.harmonics):
            p64 = p64s[h]
            nz, nr = p64.shape
            g = P[s16.plane_off[h]: s16.plane_off[h] + nz * s16.plane_row[h]].reshape(
                nz, s16.plane_row[h])[:, :nr]
            e = np.abs(g - p64) / np.maximum(p64, 1.0)
            worst_err = max(worst_err, float(e.max()))
            err_sum += float(e.sum())
            err_cells += e.size
    s32.close()
    s16.close()
    if orc is not None:
        pool.shutdown()
        orc.close()
    return {"seeds": seeds, "injected": inj, "recovered_fp32": rec32, "recovered_fp16": rec16,
            "recovery_rate_fp16": rec16 / max(inj, 1), "recovery_rate_fp32": rec32 / max(inj, 1),
            "candidate_agreement_fp16_vs_fp32": agree / max(tot32, 1),
            "max_rel_power_error_vs_fp64": worst_err,
            "mean_rel_power_error_vs_fp64": err_sum / err_cells if err_cells else None,
            "error_cells": err_cells,
            "error_metric": f"|P - P64| / max(P64, 1) over every cell of every plane of the step "
                            f"holding the first signal, for each of the {seeds} seeds (max, and mean "
                            "over all those cells)",
            "workload": "N=2^22, 3 injected signals per seed, zmax=200, 8 harmonics, L=8192, sigma=6"}


# ------------------------------------------------------------ cpu baseline
class CpuBaseline:
    """The CPU baseline: the FP32 restatement of the reference pipeline
    (oracle/cpu_fp32.py: the reference's host segment preparation, single-
    precision FFTs, its convolution / power / harmonic-sum arithmetic) over
    overlap-save steps of one 2^22-sample trial of the batched workload's
    geometry (zmax 200, 8 harmonics, L 8192), one step per task on a spawn
    process pool with one process per host core."""

    def __init__(self):
        from gpu_accelsearch_gb300.synth import synth_series
        from oracle import cpu_fp32 as F
        from oracle import oracle as O
        n = 1 << 22
        x = synth_series(n, seed=1, signals=[(0.05, 200000.25, 40.0)])
        spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
        self.w = O.deredden(spec)
        self.U = 7734
        self.numzs0 = int(O.bank_geometry(ZMAX, NUMHARM, self.U)[0, 3])
        self.cuts = np.array([O.power_cut(6.0, 1 << s) for s in range(4)])
        self.rlo = int(np.floor(np.float32(n) * np.float32(DT)))
        self.nsteps_max = O.step_count(n // 2, self.rlo, self.U)
        self.pool = F.StepPool(ZMAX, NUMHARM, self.U, self.w)
        self.cores = self.pool.processes
        self.per_step = None

    def sample(self, seconds: float):
        if self.per_step is None:  # calibrate on one step per process
            el, _ = self.pool.run([self.rlo + k * (self.U // 2) for k in range(self.cores)], self.cuts)
            self.per_step = el / self.cores
        nsteps = int(max(self.cores, min(self.nsteps_max, seconds / max(self.per_step, 1e-4))))
        startrs = [self.rlo + k * (self.U // 2) for k in range(nsteps)]
        el, nc = self.pool.run(startrs, self.cuts)
        cells = nsteps * self.U * self.numzs0
        return {"value": cells / el, "unit": "cells/s", "cores": self.cores, "kind": "port",
                "seconds": el, "candidates": nc,
                "implementation": "FP32 restatement of the reference pipeline (oracle/cpu_fp32.py): "
                                  "reference host segment preparation, scipy.fft single-precision "
                                  "FFTs, convolveSignal/generatePowers/addPowers arithmetic, "
                                  "one step per process",
                "sample": f"{nsteps} overlap-save steps of one 2^22-sample trial (zmax=200, 8 "
                          f"harmonics, L=8192, uselen=7734), {self.cores} processes, {el:.1f} s"}

    def close(self):
        self.pool.close()


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    per = max(1.0, args.cpu_seconds / 3)
    cpu = CpuBaseline()
    try:
        for _ in range(args.warmup):
            cpu.sample(per / 4)
        runs = [cpu.sample(per) for _ in range(max(1, args.steps))]
    finally:
        cpu.close()
    v = float(np.median([r["value"] for r in runs]))
    cb = dict(runs[-1])
    cb["value"] = v
    # one step = one bounded sample of the workload (the sample is in cb)
    ms = 1e3 * float(np.median([r["seconds"] for r in runs]))
    line = {"metric": METRIC, "value": v, "unit": "cells/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded N(0,1) float32 series with an injected sinusoid",
            "impl": "reference",
            "config": {"workload": "bounded sample of the batched configuration on the host: "
                                   "overlap-save steps of one 2^22-sample trial, zmax=200, "
                                   "8 harmonics, L=8192",
                       "implementation": cb["implementation"]},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------- ours
def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measure_fp32_peak(torch) -> float:
    """FP32 CUDA-core throughput of this GPU in TFLOP/s: cuBLAS FP32 GEMM
    of 8192^3 with TF32 off, best of 5 after 2 warm-ups (CUDA events)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda", dtype=torch.float32)
        b = torch.randn(n, n, device="cuda", dtype=torch.float32)
        for _ in range(2):
            c = a @ b
        best = 1e30
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            c = a @ b
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        del a, b, c
        return 2.0 * n ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def load_traffic(kernel: str, fftlen: int):
    """DRAM bytes per segment of a kernel at segment length fftlen from the
    committed ncu summary (profiles/dram_traffic_per_segment.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic_per_segment.json")) as f:
            return float(json.load(f)["by_fftlen"][str(fftlen)][kernel]["dram_bytes_per_segment"])
    except Exception:
        return None


def run_ours(args):
    import torch
    import torch.distributed as dist

    rank, local, world = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from gpu_accelsearch_gb300.search import AccelSearch

    def barrier():
        if world > 1:
            dist.barrier()

    lengths, sigs = make_batch(args.trials, seed=1000 + rank)
    series = device_series(torch, lengths, sigs, seed=2000 + rank)
    torch.cuda.synchronize()
    ptrs = [x.data_ptr() for x in series]
    from gpu_accelsearch_gb300.search import autotune
    tuned = None
    short = None if args.short_transforms < 0 else bool(args.short_transforms)
    if args.fftlen == 0 or args.chunk == 0 or args.split < 0:
        fl = (4096, 8192, 16384) if args.fftlen == 0 else (args.fftlen,)
        kw, tun, rate = autotune(ZMAX, NUMHARM, fftlens=fl, steps=1100, device=local, short_transforms=short)
        tuned = {"fftlen": kw["fftlen"], "chunk_segments": tun["chunk_segments"],
                 "plane_split": tun["plane_split"], "fused_sum": tun["fused_sum"],
                 "hsum_tile_rows": tun["hsum_tile_rows"], "sample_cells_per_s": rate}
    fftlen = args.fftlen or tuned["fftlen"]
    chunk = args.chunk or tuned["chunk_segments"]
    split = args.split if args.split >= 0 else tuned["plane_split"]
    s = AccelSearch(zmax=ZMAX, numharm=NUMHARM, fftlen=fftlen, chunk_segments=chunk, device=local,
                    short_transforms=short)
    extra = json.loads(args.tuning) if args.tuning else {}
    if tuned and "fused_sum" not in extra:
        extra["fused_sum"] = tuned["fused_sum"]
    if tuned and "hsum_tile_rows" not in extra:
        extra["hsum_tile_rows"] = tuned["hsum_tile_rows"]
    s.set_tuning(chunk_segments=chunk, plane_split=split, **extra)
    U, nz0 = s.uselen, s.harmonics[0].numzs
    nseg = sum(s.step_count(n, DT) for n in lengths)
    cells = nseg * U * nz0
    # plane cells per segment (mean row width over the step phases ~ plane_width - 1)
    sub_cells = sum(h.numzs * (h.plane_width - 1) for h in s.harmonics[1:])
    bytes_per_cell = 8.0 * (sub_cells + U * nz0) / (U * nz0)

    for _ in range(args.warmup):
        s.search(ptrs, DT, on_device=True, nsamples=lengths)
    torch.cuda.synchronize()

    # ---- value: device-resident inputs
    s.reset_stats()
    s.profile(True)
    clk = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    clk.start()
    t0 = time.perf_counter()
    ncand = 0
    for _ in range(args.steps):
        ncand = s.search(ptrs, DT, on_device=True, nsamples=lengths)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    clocks = clk.stop()
    barrier()
    st = s.stats()
    s.profile(False)
    wall = el
    el_t = torch.tensor([st["search_ms"] / 1e3], device="cuda")  # CUDA-event device time
    if world > 1:
        dist.all_reduce(el_t, op=dist.ReduceOp.MAX)
    el = float(el_t.item())
    value = cells * args.steps * world / el

    # ---- e2e: pinned host series through the C ABI, host wall clock from
    # the call to its return (copies in, search, candidate read-back and the
    # host's conversion and sort of the candidate list)
    e2e = None
    if not args.no_e2e:
        host = [x.cpu().pin_memory() for x in series]
        hptrs = [h.data_ptr() for h in host]
        s.search_ptrs(hptrs, lengths, DT, on_device=False)  # warm
        barrier()
        torch.cuda.synchronize()
        s.reset_stats()
        nc = 0
        clk2 = Clocks(local)
        clk2.start()
        t2 = time.perf_counter()
        for _ in range(args.steps):
            nc = s.search_ptrs(hptrs, lengths, DT, on_device=False)
        torch.cuda.synchronize()
        wall2 = time.perf_counter() - t2
        clocks_e2e = clk2.stop()
        dev2 = s.stats()["search_ms"] / 1e3
        barrier()
        el2_t = torch.tensor([wall2, dev2], device="cuda")
        if world > 1:
            dist.all_reduce(el2_t, op=dist.ReduceOp.MAX)
        wall2, dev2 = float(el2_t[0].item()), float(el2_t[1].item())
        e2e = {"value": cells * args.steps * world / wall2, "unit": "cells/s",
               "h2d_bytes_per_step": int(sum(lengths) * 4),
               "d2h_bytes_per_step": int(16 + 16 * nc),
               "timing": "host wall clock around accel_search (pinned host series in, candidate "
                         "list out, host conversion and sort included); max over ranks",
               "wall_ms_per_step": 1e3 * wall2 / args.steps,
               "device_event_ms_per_step": 1e3 * dev2 / args.steps,
               "clocks": clocks_e2e}

    # ---- plain per-trial path, two ways: (a) the reference's control flow,
    # one overlap-save step per launch group, one 2^22 trial; (b) one 2^22
    # trial per search at the tuned launch-group size and layout -- what
    # batching across trials adds beyond filling the launch groups
    plain = plain_trial = None
    if not args.no_plain and rank == 0:
        xs = device_series(torch, [1 << 22], [None], seed=7)

        def time_trial(search, reps=3):
            search.search([xs[0].data_ptr()], DT, on_device=True, nsamples=[1 << 22])
            torch.cuda.synchronize()
            search.reset_stats()
            for _ in range(reps):
                search.search([xs[0].data_ptr()], DT, on_device=True, nsamples=[1 << 22])
            torch.cuda.synchronize()
            n1 = search.step_count(1 << 22, DT)
            return n1, n1 * search.uselen * search.harmonics[0].numzs * reps / (search.stats()["search_ms"] / 1e3)

        p = AccelSearch(zmax=ZMAX, numharm=NUMHARM, fftlen=FFTLEN, chunk_segments=1, device=local,
                        short_transforms=short)
        pn, pv = time_trial(p)
        p.close()
        plain = {"value": pv, "unit": "cells/s",
                 "workload": "one 2^22-sample trial, one overlap-save step per launch group "
                             f"({pn} steps, L={FFTLEN}): the reference's step-at-a-time control flow"}
        # the batch itself, one trial per search call (device-resident
        # series, the batched search's tuned launch shape)
        q = AccelSearch(zmax=ZMAX, numharm=NUMHARM, fftlen=fftlen, chunk_segments=chunk, device=local,
                        short_transforms=short)
        q.set_tuning(chunk_segments=chunk, plane_split=split, **extra)
        for i in range(min(4, len(ptrs))):
            q.search([ptrs[i]], DT, on_device=True, nsamples=[lengths[i]])
        torch.cuda.synchronize()
        q.reset_stats()
        t3 = time.perf_counter()
        for i in range(len(ptrs)):
            q.search([ptrs[i]], DT, on_device=True, nsamples=[lengths[i]])
        torch.cuda.synchronize()
        wall3 = time.perf_counter() - t3
        dev3 = q.stats()["search_ms"] / 1e3
        q.close()
        plain_trial = {"value": cells / dev3, "unit": "cells/s", "wall_value": cells / wall3,
                       "workload": f"the same {len(ptrs)} trials, one accel_search call per trial "
                                   f"(launch groups of {chunk} segments, L={fftlen}): what searching "
                                   "the trials together adds"}

    if rank != 0:
        s.close()
        if world > 1:
            dist.destroy_process_group()
        return

    peak, peak_kind = load_peaks()
    k = st["kinds"]
    # algorithmic bytes per kernel: k_plane writes each plane cell it
    # produces once (4 B); k_hsum reads every plane cell once (4 B); in the
    # fused layout k_fund_sum reads the sub-harmonic cells once and the
    # fundamental plane never leaves the chip.
    segs = st["segments"]
    fused = s.tuning()["fused_sum"]
    fund_cells = U * nz0
    cells_by_kind = {"plane": sub_cells + (0 if fused else fund_cells),
                     "hsum": sub_cells + fund_cells, "fund": sub_cells}
    per_kernel = {}
    for name in ("plane", "hsum", "fund"):
        ms = k[name]["ms"]
        if ms > 0:
            b = 4.0 * cells_by_kind[name] * segs
            per_kernel[name] = {"launches": k[name]["launches"], "ms": ms,
                                "bytes_per_launch": b / max(k[name]["launches"], 1),
                                "achieved": b / (ms / 1e3) / 1e9}
    dom = max(per_kernel, key=lambda n: per_kernel[n]["ms"]) if per_kernel else None
    names = {"plane": "k_plane (correlate + inverse FFT + |X|^2 power planes)",
             "hsum": "k_hsum_tile (harmonic sum + threshold over shared-memory tiles)",
             "fund": "k_fund_sum (fundamental plane fused with harmonic sum + threshold)"}
    tr = load_traffic(dom, fftlen) if dom else None
    roofline = None
    import math
    # algorithmic FP32 work of one segment's plane rows: two M-point inverse
    # FFTs per template at the radix-2 count 5 M log2 M, plus the template
    # products (6 flops per point) and the powers (3 flops per point)
    flops_seg = sum(h.numzs * (2 * 5 * (h.fftlen // 2) * math.log2(h.fftlen // 2) + 18 * (h.fftlen // 2))
                    for h in s.harmonics)
    fp32_peak = measure_fp32_peak(torch)
    if dom:
        pk = per_kernel[dom]
        hbm_axis = {"achieved": pk["achieved"], "peak": peak, "unit": "GB/s", "frac": pk["achieved"] / peak,
                    "peak_source": peak_kind, "algorithmic_bytes_per_launch": pk["bytes_per_launch"],
                    "note": "algorithmic bytes (4 B per plane cell moved) per launch / mean CUDA-event "
                            "time of its launches in the timed region"}
        traffic = (tr * segs / max(pk["launches"], 1)) if tr else None
        if dom in ("plane", "fund"):
            # what bounds the plane kernel (ncu: issue slots 68 %, FP32 pipe
            # 52 %, L1/shared 69 %, DRAM 19 %) is its FP32 work, not HBM
            achieved_tf = flops_seg * segs / (k[dom]["ms"] / 1e3) / 1e12
            roofline = {"bound": "fp32", "kernel": names[dom], "achieved": achieved_tf,
                        "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved_tf / fp32_peak,
                        "peak_source": "measured in this run: cuBLAS FP32 GEMM 8192^3 with TF32 off "
                                       "(no FP32 figure in MEASURED_PEAKS.json)",
                        "flops_per_segment": flops_seg, "traffic": traffic, "hbm": hbm_axis,
                        "note": "achieved = algorithmic FP32 flops per launch (radix-2 FFT count) / "
                                "mean CUDA-event time of its launches in the timed region"}
        else:
            roofline = dict(hbm_axis, bound="hbm", kernel=names[dom], traffic=traffic)
        roofline["per_kernel"] = {n: {"achieved_GBs": round(v["achieved"], 1), "frac_hbm": round(v["achieved"] / peak, 4)}
                                  for n, v in per_kernel.items()}
    step_roofline = {"bytes_per_cell": bytes_per_cell,
                     "achieved": value / world * bytes_per_cell / 1e9, "peak": peak,
                     "unit": "GB/s", "frac": value / world * bytes_per_cell / 1e9 / peak,
                     "note": "every plane written once and read once per fundamental cell"}
    tot_ms = max(sum(x["ms"] for x in k.values()), 1e-9)
    kern = {name: {"launches": v["launches"], "ms": round(v["ms"], 3),
                   "share": round(v["ms"] / tot_ms, 4)} for name, v in k.items() if v["launches"]}
    cb = None
    if args.cpu_seconds > 0:
        cpu = CpuBaseline()
        try:
            cb = cpu.sample(args.cpu_seconds)
        finally:
            cpu.close()
    dedisp = run_dedisperse(local) if args.serving_seconds > 0 else None
    serving = (run_serving(args.serving_seconds, local, chunk=args.serving_chunk, lengths=args.serving_lengths,
                           max_chunk=args.serving_max_chunk)
               if args.serving_seconds > 0 else None)
    # the same stream at half the rate: latency when the GPU is not saturated
    serving_half = (run_serving(args.serving_seconds, local, rate=100.0, chunk=args.serving_chunk,
                                lengths=args.serving_lengths, max_chunk=args.serving_max_chunk)
                    if args.serving_seconds > 0 else None)
    precision = precision_report(args.precision_seeds, local) if args.precision_seeds > 0 else None
    line = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "wall_ms_per_step": 1e3 * wall / args.steps, "timing": "CUDA events on the library stream, "
        "first input copy to last candidate read-back; max over ranks",
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded N(0,1) float32 series (torch Philox), 10% with one "
                "injected accelerated sinusoid",
        "config": {"workload": f"batched: {args.trials} DM trials per GPU, lengths uniform in "
                               "{2^20, 2^21, 2^22, 3*2^20}, dt=64us, zmax=200, 8 harmonics, "
                               f"L={fftlen} (uselen {U}) chosen by the autotuner, sigma=6",
                   "segments_per_step": nseg, "cells_per_step": cells,
                   "fftlen": fftlen, "uselen": U, "tuning": s.tuning(), "autotuner": tuned,
                   "transform_lengths": [h.fftlen for h in s.harmonics],
                   "l2": f"inputs ({sum(lengths) * 4 / 1e9:.2f} GB of series per GPU) larger "
                         "than L2; no flush",
                   "parallelism": f"trial-sharded replicas x{world}"},
        "roofline": roofline, "step_roofline": step_roofline, "kernels": kern,
        "cpu_baseline": cb, "e2e": e2e, "gpu_launches": st["launches"], "clocks": clocks,
        "plain": plain,
        "batched_over_plain": (value / world / plain["value"]) if plain else None,
        "plain_per_trial": plain_trial,
        "batched_over_plain_per_trial": (value / world / plain_trial["value"]) if plain_trial else None,
        "candidates_per_step": ncand,
        "serving": serving, "serving_half_load": serving_half, "dedisperse": dedisp,
        "precision_fp16": precision,
    }
    print(json.dumps(line), flush=True)
    s.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
