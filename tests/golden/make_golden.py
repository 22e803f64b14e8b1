"""Generate tests/golden/reference_pins.json from the reference's own code.

Run from the repository root, in a container that has the reference sources:

    make -C oracle/ref -j            # builds oracle/_ref/libref_u<USELEN>.so
    python tests/golden/make_golden.py

The libraries are the reference's host code (bpd_math.c, bpd_noise.c,
bpd_fresnl.c, bpd_subharmonics.cu, bpd_search.cu, ...) compiled from its
sources by oracle/ref/Makefile.  Every value in the JSON file was produced by
that code; tests/test_oracle_pins.py checks the CPU oracle against it.
Inputs are seeded numpy streams; their SHA-256 is stored so that a change of
generator shows up as an input mismatch rather than a parity failure.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from gpu_accelsearch_gb300.synth import synth_series, synth_red_spectrum  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "reference_pins.json")
FP, DP, IP = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def reflib(uselen: int):
    path = os.path.join(ROOT, "oracle", "_ref", f"libref_u{uselen}.so")
    L = C.CDLL(path)
    L.ref_uselen.restype = C.c_int
    L.ref_rsqrt.restype, L.ref_rsqrt.argtypes = C.c_float, [C.c_float]
    L.ref_fast_median.restype, L.ref_fast_median.argtypes = C.c_float, [FP, C.c_int]
    L.ref_fresnl.argtypes = [C.c_double, DP, DP]
    L.ref_z_halfwidth.restype, L.ref_z_halfwidth.argtypes = C.c_int, [C.c_double]
    L.ref_calc_required_z.restype = C.c_int
    L.ref_calc_required_z.argtypes = [C.c_double, C.c_double]
    L.ref_calc_required_r.restype = C.c_double
    L.ref_calc_required_r.argtypes = [C.c_double, C.c_double]
    L.ref_fft_length.restype = C.c_int
    L.ref_fft_length.argtypes = [C.c_int, C.c_int, C.c_int]
    L.ref_deredden.argtypes = [FP, C.c_uint]
    L.ref_r_response.argtypes = [C.c_double, C.c_int, C.c_int, FP]
    L.ref_z_response.argtypes = [C.c_double, C.c_int, C.c_double, C.c_int, FP]
    L.ref_create_bank.restype, L.ref_create_bank.argtypes = C.c_void_p, [C.c_int, C.c_int]
    L.ref_bank_info.argtypes = [C.c_void_p, C.c_int, IP]
    L.ref_bank_templates.restype = FP
    L.ref_bank_templates.argtypes = [C.c_void_p, C.c_int]
    L.ref_step_ffdot.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double,
                                 IP, DP]
    L.ref_step_data.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double,
                                FP, C.c_long, FP]
    assert L.ref_uselen() == uselen
    return L


def fp(a):
    return a.ctypes.data_as(FP)


# Bank / search configurations: (zmax, numharm, uselen)
BANKS = [(50, 4, 1914), (200, 8, 7734), (200, 8, 3638), (200, 8, 15926), (300, 8, 32000),
         (100, 8, 7734), (50, 8, 3638)]


def main():
    pins: dict = {"generator": "numpy PCG64 (gpu_accelsearch_gb300/synth.py)"}
    L = reflib(1914)

    # scalar host math
    xs = np.linspace(0.0, 40.0, 4001, dtype=np.float32)
    pins["rsqrt"] = {"x_sha": sha(xs),
                     "y_sha": sha(np.array([L.ref_rsqrt(float(x)) for x in xs], np.float32))}
    fx = np.concatenate([np.linspace(-60.0, 60.0, 2401), [-40000.0, 36975.0, 1e-9, 1.6]])
    fs, fc = C.c_double(), C.c_double()
    sc = []
    for x in fx:
        L.ref_fresnl(float(x), C.byref(fs), C.byref(fc))
        sc.append((fs.value, fc.value))
    pins["fresnl"] = {"x": fx.tolist(), "sc": sc}
    pins["z_halfwidth"] = {str(z): L.ref_z_halfwidth(float(z)) for z in range(-1200, 1201, 2)}
    req = []
    for (h, H) in [(1, 1), (1, 2), (1, 4), (3, 4), (1, 8), (3, 8), (5, 8), (7, 8),
                   (1, 16), (15, 16)]:
        f = h / H
        for z in (-300, -200, -150, -100, -51, -50, 0, 2, 50, 77, 200, 300):
            req.append(["z", h, H, z, L.ref_calc_required_z(f, float(z))])
        for r in (0.0, 16.0, 957.5, 20000.25, 131071.5, 2097151.0):
            req.append(["r", h, H, r, L.ref_calc_required_r(f, r)])
    pins["calc_required"] = req

    # responses: sha of the float32 bytes, per z
    resp = {}
    for z in (0, 2, -2, 26, -26, 50, -50, 76, -150, 200, -200, 300, -300):
        hw = L.ref_z_halfwidth(float(z))
        out = np.zeros(8 * hw, np.float32)
        L.ref_z_response(0.0, 2, float(z), 4 * hw, fp(out))
        resp[str(z)] = {"numkern": 4 * hw, "sha": sha(out), "head": out[:8].tolist()}
    out = np.zeros(2 * 64, np.float32)
    L.ref_r_response(0.25, 2, 64, fp(out))
    resp["r_response_0.25_64"] = {"sha": sha(out)}
    pins["responses"] = resp

    # median selection (destructive in the reference; give it a copy)
    med = []
    rng = np.random.default_rng(7)
    for n in (1, 2, 3, 6, 11, 200, 1000, 2067, 4096):
        a = rng.exponential(1.0, n).astype(np.float32)
        if n > 10:
            a[: n // 5] = a[n // 3]  # duplicates
        b = a.copy()
        med.append({"n": n, "a_sha": sha(a), "seed": 7, "m": float(L.ref_fast_median(fp(b), n))})
    pins["median_seeded"] = med

    # whitening of a seeded red spectrum (numbins = 2^17, the N=2^18 case)
    spec = synth_red_spectrum(1 << 17, seed=11)
    w = spec.copy()
    L.ref_deredden(fp(w.view(np.float32)), w.size)
    pins["deredden"] = {"numbins": int(spec.size), "seed": 11, "in_sha": sha(spec),
                        "out_sha": sha(w), "head": w.view(np.float32)[:16].tolist()}
    # short spectra whose last block slope drives the extrapolated tail level
    # below zero (5220 bins: NaN at the end) beside ordinary ones
    tails = []
    for numbins in (3000, 4184, 5220):
        spec = synth_red_spectrum(numbins + 1, seed=numbins)[:numbins]
        w = spec.copy()
        L.ref_deredden(fp(w.view(np.float32)), w.size)
        f = w.view(np.float32)
        tails.append({"numbins": numbins, "seed": numbins, "in_sha": sha(spec), "out_sha": sha(w),
                      "nan_floats": np.nonzero(np.isnan(f))[0].tolist()})
    pins["deredden_tails"] = tails

    # banks: geometry + time-domain templates
    banks = []
    for (zmax, numharm, uselen) in BANKS:
        R = reflib(uselen)
        stages = int(np.log2(numharm)) + 1
        b = R.ref_create_bank(stages, zmax)
        nh = 1 << (stages - 1)
        hs = []
        for h in range(nh):
            info = np.zeros(6, np.int32)
            R.ref_bank_info(b, h, info.ctypes.data_as(IP))
            numzs, L_h = int(info[3]), int(info[4])
            tp = np.ctypeslib.as_array(R.ref_bank_templates(b, h), shape=(numzs * L_h * 2,))
            hs.append({"info": info.tolist(), "templates_sha": sha(tp.astype(np.float32))})
        banks.append({"zmax": zmax, "numharm": numharm, "uselen": uselen, "harmonics": hs})
    pins["banks"] = banks

    # step geometry and segment data on a whitened synthetic series
    steps = []
    for (zmax, numharm, uselen, nlog2, dt, sample_steps) in [
            (50, 4, 1914, 18, 64e-6, None), (200, 8, 7734, 22, 64e-6, [0, 1, 2, 270, 540, 541])]:
        R = reflib(uselen)
        stages = int(np.log2(numharm)) + 1
        b = R.ref_create_bank(stages, zmax)
        n = 1 << nlog2
        x = synth_series(n, seed=1000 + nlog2, signals=[(0.05, 20000.25, 40.0)])
        spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)
        numbins = n // 2
        w = spec[:numbins].copy()
        R.ref_deredden(fp(w.view(np.float32)), numbins)
        rlo = int(np.floor(1.0 * float(np.float32(n) * np.float32(dt))))
        half = uselen // 2
        nsteps = 0
        s = rlo
        while s + half < numbins:
            nsteps += 1
            s += half
        idx = list(range(nsteps)) if sample_steps is None else sample_steps
        nh = 1 << (stages - 1)
        total = 0
        for h in range(nh):
            info = np.zeros(6, np.int32)
            R.ref_bank_info(b, h, info.ctypes.data_as(IP))
            total += int(info[4])
        recs = []
        for k in idx:
            startr = float(rlo + k * half)
            lastr = startr + half - 0.5
            oi = np.zeros(6 * nh, np.int32)
            orhi = np.zeros(nh, np.float64)
            R.ref_step_ffdot(b, stages, startr, lastr, float(-zmax), oi.ctypes.data_as(IP),
                             orhi.ctypes.data_as(DP))
            data = np.zeros(2 * total, np.float32)
            R.ref_step_data(b, stages, startr, lastr, float(-zmax), fp(w.view(np.float32)),
                            numbins, fp(data))
            recs.append({"step": k, "startr": startr, "ffdot": oi.tolist(),
                         "rhi": orhi.tolist(), "data_sha": sha(data)})
        steps.append({"zmax": zmax, "numharm": numharm, "uselen": uselen, "nlog2": nlog2,
                      "dt": dt, "series_seed": 1000 + nlog2, "series_sha": sha(x),
                      "whitened_sha": sha(w), "rlo": rlo, "nsteps": nsteps, "steps": recs})
    pins["steps"] = steps

    with open(OUT, "w") as f:
        json.dump(pins, f, indent=0)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
