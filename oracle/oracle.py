"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module; the product library never does.  The C side
(accel_oracle.c) restates the reference algorithm: host numerics bit-for-bit,
the cuFFT/kernel stages in FP64.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
HINFO = 7  # harmnum, maxharm, zmax_h, numzs, fftlen, hw0, zlo


class OrcCand(C.Structure):
    _fields_ = [("step", C.c_int), ("ridx", C.c_int), ("zidx", C.c_int),
                ("numharm", C.c_int), ("power", C.c_double)]


def build() -> str:
    """Compile liboracle.so if it is missing or older than its sources."""
    src = [os.path.join(_HERE, f) for f in ("accel_oracle.c", "accel_oracle.h")]
    if (not os.path.exists(_LIB)
            or max(os.path.getmtime(s) for s in src) > os.path.getmtime(_LIB)):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        fp, dp, ip = (C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int))
        sig = {
            "orc_rsqrt_magic": (C.c_float, [C.c_float]),
            "orc_rsqrt_norm": (C.c_float, [C.c_float]),
            "orc_set_exact_rsqrt": (None, [C.c_int]),
            "orc_select_lower_median": (C.c_float, [fp, C.c_int]),
            "orc_next_pow2": (C.c_longlong, [C.c_longlong]),
            "orc_fresnl": (C.c_int, [C.c_double, dp, dp]),
            "orc_z_halfwidth": (C.c_int, [C.c_double]),
            "orc_calc_required_z": (C.c_int, [C.c_double, C.c_double]),
            "orc_calc_required_r": (C.c_double, [C.c_double, C.c_double]),
            "orc_fft_length": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int]),
            "orc_r_response": (None, [C.c_double, C.c_int, C.c_int, fp]),
            "orc_z_response": (None, [C.c_double, C.c_int, C.c_double, C.c_int, fp]),
            "orc_wrapped_template": (None, [C.c_int, C.c_int, fp]),
            "orc_deredden": (None, [fp, C.c_uint, C.c_int, C.c_int]),
            "orc_bank_geometry": (C.c_int, [C.c_int, C.c_int, C.c_int, ip]),
            "orc_step_ffdot": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                      C.c_double, ip, dp, ip, ip]),
            "orc_segment_data": (C.c_int, [fp, C.c_long, C.c_int, C.c_double, C.c_int,
                                           C.c_int, fp]),
            "orc_step_count": (C.c_long, [C.c_long, C.c_long, C.c_int]),
            "orc_create": (C.c_void_p, [C.c_int, C.c_int, C.c_int]),
            "orc_destroy": (None, [C.c_void_p]),
            "orc_num_harmonics": (C.c_int, [C.c_void_p]),
            "orc_run_steps": (C.c_long, [C.c_void_p, fp, C.c_long, C.c_long, C.c_long,
                                         C.c_long, dp, dp, C.POINTER(OrcCand), C.c_long,
                                         C.c_int]),
            "orc_harmonic_plane": (C.c_int, [C.c_void_p, fp, C.c_long, C.c_double, C.c_int,
                                             dp, C.c_int]),
            "orc_power_cut": (C.c_double, [C.c_double, C.c_int, C.c_double]),
            "orc_fft": (None, [dp, C.c_int, C.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


# ---------------------------------------------------------------- scalars
def rsqrt_magic(x: float) -> float:
    return lib().orc_rsqrt_magic(x)


def set_exact_rsqrt(on: bool) -> None:
    """Switch the oracle's normalisations (deredden, segment norms) between
    the reference's magic-constant rsqrt (default) and IEEE 1/sqrtf -- the
    GPU build's exact_rsqrt option."""
    lib().orc_set_exact_rsqrt(int(bool(on)))


def rsqrt_norm(x: float) -> float:
    return lib().orc_rsqrt_norm(x)


def lower_median(a) -> float:
    a = np.ascontiguousarray(a, dtype=np.float32)
    return lib().orc_select_lower_median(_fp(a), a.size)


def fresnl(x: float):
    s, c = C.c_double(), C.c_double()
    lib().orc_fresnl(x, C.byref(s), C.byref(c))
    return s.value, c.value


def z_halfwidth(z: float) -> int:
    return lib().orc_z_halfwidth(z)


def calc_required_z(f: float, z: float) -> int:
    return lib().orc_calc_required_z(f, z)


def calc_required_r(f: float, r: float) -> float:
    return lib().orc_calc_required_r(f, r)


def fft_length(numharm: int, harmnum: int, zmax: int, uselen: int) -> int:
    return lib().orc_fft_length(numharm, harmnum, zmax, uselen)


def power_cut(sigma: float, numharm: int, numindep: float = 1.0) -> float:
    return lib().orc_power_cut(sigma, numharm, numindep)


def step_count(highest_bin: int, rlo: int, uselen: int) -> int:
    return lib().orc_step_count(highest_bin, rlo, uselen)


# ---------------------------------------------------------------- arrays
def z_response(z: float, numkern: int, roffset: float = 0.0, numbetween: int = 2):
    out = np.zeros(2 * numkern, np.float32)
    lib().orc_z_response(roffset, numbetween, z, numkern, _fp(out))
    return out.view(np.complex64)


def r_response(numkern: int, roffset: float = 0.0, numbetween: int = 2):
    out = np.zeros(2 * numkern, np.float32)
    lib().orc_r_response(roffset, numbetween, numkern, _fp(out))
    return out.view(np.complex64)


def wrapped_template(fftlen: int, z: int):
    out = np.zeros(2 * fftlen, np.float32)
    lib().orc_wrapped_template(fftlen, z, _fp(out))
    return out.view(np.complex64)


def deredden(spec, initialbuflen: int = 6, maxbuflen: int = 200):
    """Whitening of a complex64 spectrum; returns a new array (numbins = len)."""
    s = np.array(spec, dtype=np.complex64, copy=True)
    f = s.view(np.float32)
    lib().orc_deredden(_fp(f), s.size, initialbuflen, maxbuflen)
    return s


def bank_geometry(zmax: int, numharm: int, uselen: int):
    info = np.zeros(16 * HINFO, np.int32)
    n = lib().orc_bank_geometry(zmax, numharm, uselen, _ip(info))
    return info[: n * HINFO].reshape(n, HINFO)


def step_ffdot(harmnum, maxharm, zmax, uselen, startr, lastr):
    rlo, zlo, numrs = C.c_int(), C.c_int(), C.c_int()
    rhi = C.c_double()
    lib().orc_step_ffdot(harmnum, maxharm, zmax, uselen, startr, lastr, C.byref(rlo),
                         C.byref(rhi), C.byref(zlo), C.byref(numrs))
    return rlo.value, rhi.value, zlo.value, numrs.value


def segment_data(wspec, rlo, rhi, hw0, fftlen):
    w = np.ascontiguousarray(wspec, dtype=np.complex64)
    out = np.zeros(2 * fftlen, np.float32)
    rc = lib().orc_segment_data(_fp(w.view(np.float32)), w.size, rlo, rhi, hw0, fftlen,
                                _fp(out))
    if rc != 0:
        raise ValueError("segment length mismatch")
    return out.view(np.complex64)


class Oracle:
    """FP64 search over a template bank of (zmax, numharm, uselen)."""

    def __init__(self, zmax: int, numharm: int, uselen: int):
        self.zmax, self.numharm, self.uselen = zmax, numharm, uselen
        self._h = lib().orc_create(zmax, numharm, uselen)
        self.geom = bank_geometry(zmax, numharm, uselen)
        self.nh = len(self.geom)
        self.nstages = sum(1 for h in range(self.nh) if ((h + 1) & h) == 0)

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run_steps(self, wspec, rlo, step0, nsteps, powcut=None, want_planes=False,
                  cap=1 << 20, nthreads=None):
        """Returns (candidates structured array, stage planes or None, total count)."""
        w = np.ascontiguousarray(wspec, dtype=np.complex64)
        numzs0 = int(self.geom[0, 3])
        planes = None
        if want_planes:
            planes = np.zeros((nsteps, self.nstages, numzs0, self.uselen), np.float64)
        pc = None
        if powcut is not None:
            pc = np.ascontiguousarray(powcut, dtype=np.float64)
        cands = (OrcCand * max(cap, 1))()
        nthreads = nthreads or os.cpu_count() or 1
        n = lib().orc_run_steps(self._h, _fp(w.view(np.float32)), w.size, rlo, step0, nsteps,
                                _dp(pc) if pc is not None else None,
                                _dp(planes) if planes is not None else None, cands, cap,
                                nthreads)
        m = min(n, cap)
        arr = np.zeros(m, dtype=[("step", "i4"), ("ridx", "i4"), ("zidx", "i4"),
                                 ("numharm", "i4"), ("power", "f8")])
        for k in range(m):
            c = cands[k]
            arr[k] = (c.step, c.ridx, c.zidx, c.numharm, c.power)
        return arr, planes, n

    def harmonic_plane(self, wspec, startr, h, wcap=None):
        w = np.ascontiguousarray(wspec, dtype=np.complex64)
        numzs = int(self.geom[h, 3])
        wcap = wcap or int(self.geom[h, 4])
        plane = np.zeros((numzs, wcap), np.float64)
        n = lib().orc_harmonic_plane(self._h, _fp(w.view(np.float32)), w.size, startr, h,
                                     _dp(plane), wcap)
        return plane[:, :n]


def fft64(x, sign=-1):
    a = np.array(x, dtype=np.complex128, copy=True)
    lib().orc_fft(_dp(a.view(np.float64)), a.size, sign)
    return a


def sift(cands, min_dr=15.0, maxharm=8, harm_dr=1.0):
    """Candidate sifting restated with plain loops (small cases only): per
    trial, by sigma (then power, r, z, numharm); drop a candidate strictly
    closer than min_dr in r to a kept one; then drop one within harm_dr of
    (a/b) times a stronger survivor's r, 1 <= a, b <= maxharm, a != b, a/b
    in lowest terms.  Returns the survivors in that order."""
    from math import gcd
    ratios = [(a, b) for a in range(1, maxharm + 1) for b in range(1, maxharm + 1)
              if a != b and gcd(a, b) == 1]
    order = sorted(range(len(cands)), key=lambda k: (
        int(cands[k]["trial"]), -float(cands[k]["sigma"]), -float(cands[k]["power"]),
        float(cands[k]["r"]), float(cands[k]["z"]), int(cands[k]["numharm"])))
    out = []
    trials = sorted({int(c["trial"]) for c in cands})
    for t in trials:
        group = []
        for k in order:
            c = cands[k]
            if int(c["trial"]) != t:
                continue
            if min_dr > 0 and any(abs(float(g["r"]) - float(c["r"])) < min_dr for g in group):
                continue
            group.append(c)
        final = []
        for c in group:
            harmonic = maxharm > 1 and any(
                abs(float(c["r"]) - a / b * float(f["r"])) <= harm_dr
                for f in final for a, b in ratios)
            if not harmonic:
                final.append(c)
        out.extend(final)
    return out


def harmonic_power(wspec, r, z):
    """|sum_j X[j] conj(F(r - j - z/2; z))|^2 over the 2 hw(z) bins j in
    [ceil(r - hw), ceil(r + hw)): the plane kernels' correlation at any
    (r, z), with F from the restated generate_z_response (numbetween 1,
    offset chosen so that its samples fall on x = r - j - z/2)."""
    import math
    hw = z_halfwidth(z)
    j0 = math.ceil(r - hw)
    # samples x = r - j - z/2 for j = j0 .. j0 + 2hw - 1 are 2hw consecutive
    # elements of a 2hw+2 point response with its offset in [0, 1) (the range
    # the reference's routine is written for), starting at element s
    d = r - j0
    off = d - math.floor(d)
    s = int(round(off + hw + 1 - d))
    resp = z_response(z, 2 * hw + 2, roffset=off, numbetween=1)[s: s + 2 * hw]
    resp = resp.astype(np.complex128)
    j = np.arange(j0, j0 + 2 * hw)
    ok = (j >= 0) & (j < len(wspec))
    x = np.zeros(2 * hw, np.complex128)
    x[ok] = wspec[j[ok]]
    a = np.sum(x * np.conj(resp))
    return float(a.real * a.real + a.imag * a.imag)


def step_norms(wspec, zmax, bank_numharm, uselen, rlo, step, numharm):
    """Squared segment normalisation of harmonics k/numharm (k = 1..numharm)
    in overlap-save step `step` of a trial whose first bin is rlo: the
    magic rsqrt of the lower median of |X|^2 over the segment's numdata bins
    divided by ln 2 (bpd_search.cu:130-184)."""
    from math import gcd, ceil, log
    geom = bank_geometry(zmax, bank_numharm, uselen)
    startr = rlo + step * (uselen // 2)
    out = []
    for k in range(1, numharm + 1):
        g = gcd(k, numharm)
        p, q = k // g, numharm // g
        row = [rw for rw in geom if int(rw[0]) == p and int(rw[1]) == q][0]
        hw0, fftlen = int(row[5]), int(row[4])
        rl, rh, _, _ = step_ffdot(p, q, zmax, uselen, float(startr), startr + uselen // 2 - 0.5)
        lobin = rl - hw0
        numdata = min(int(ceil(rh)) + hw0 - lobin + 1, fftlen // 2)
        idx = np.arange(lobin, lobin + numdata)
        v = np.zeros(numdata, np.complex64)
        ok = (idx >= 0) & (idx < len(wspec))
        v[ok] = wspec[idx[ok]]
        pw = (v.real * v.real + v.imag * v.imag).astype(np.float32)
        nrm = rsqrt_norm(float(np.float64(lower_median(pw)) / log(2.0)))
        out.append(float(nrm) * float(nrm))
    return out


def optimize(wspec, r, z, numharm, norms, refine=True):
    """Candidate refinement restated: the summed power of harmonics
    k r/numharm, k z/numharm (k = 1..numharm; harmonic k scaled by norms[k-1])
    maximised over three nested 5 x 5 grids (steps 1/4, 1/16, 1/64 in r;
    1, 1/4, 1/16 in z), the centre kept unless a point is strictly larger.
    Returns (r, z, power, powers per harmonic)."""
    def summed(rr, zz):
        return sum(norms[k - 1] * harmonic_power(wspec, rr * k / numharm, zz * k / numharm)
                   for k in range(1, numharm + 1))
    if refine:
        for dr, dz in ((0.25, 1.0), (1 / 16, 0.25), (1 / 64, 1 / 16)):
            pts = [(r + (g // 5 - 2) * dr, z + (g % 5 - 2) * dz) for g in range(25)]
            p = [summed(a, b) for a, b in pts]
            best = 12
            for g in range(25):
                if p[g] > p[best]:
                    best = g
            r, z = pts[best]
    hp = [norms[k - 1] * harmonic_power(wspec, r * k / numharm, z * k / numharm)
          for k in range(1, numharm + 1)]
    return r, z, sum(hp), hp


# ------------------------------------------------------------ dedispersion
# Not part of the reference (it starts from dedispersed series).  The
# restatement follows the standard cold-plasma dispersion delay
# (Lorimer & Kramer, Handbook of Pulsar Astronomy, eq. 5.1: 4.148808e3 s
# MHz^2 pc^-1 cm^3 x DM x (f^-2 - f_ref^-2)) and the direct method of
# incoherent dedispersion; parity for this stage is against this
# restatement only (no reference implementation exists to pin it).
DISP_CONST = 4.148808e3


def dm_delays(nchan, f_top_mhz, chan_bw_mhz, tsamp, dms):
    """int32[ndm][nchan] delays in samples, rounded half up, relative to the
    highest channel frequency (the evaluation order of the library's host
    code, operation by operation in double precision)."""
    f = f_top_mhz + np.arange(nchan, dtype=np.float64) * chan_bw_mhz
    f_ref = max(f_top_mhz, float(f[-1]))
    inv_ref2 = 1.0 / (f_ref * f_ref)
    dm = np.asarray(dms, dtype=np.float32).astype(np.float64)[:, None]
    v = np.floor(DISP_CONST * dm * (1.0 / (f * f) - inv_ref2) / tsamp + 0.5)
    return v.astype(np.int32)


def dedisperse(fb, delays, nout):
    """float32[ndm][nout]: for each DM trial the channels of fb (float32
    [nchan][nsamp]) shifted by their delays and added in channel order with
    float32 rounding after every addition."""
    fb = np.asarray(fb, dtype=np.float32)
    ndm, nchan = delays.shape
    out = np.zeros((ndm, nout), np.float32)
    for d in range(ndm):
        acc = np.zeros(nout, np.float32)
        for c in range(nchan):
            s = int(delays[d, c])
            acc += fb[c, s:s + nout]
        out[d] = acc
    return out
