"""Generate tests/golden/reference_planes.npz: power planes and harmonic
stage sums produced by the reference's own code for single overlap-save
steps, the golden planes the GPU tests compare the fused path against.

Run from the repository root, in a container that has the reference sources:

    make -C oracle/ref -j REF=<reference checkout>
    python tests/golden/make_plane_golden.py

Stage by stage, one step of AccelSearch.cu:209-245:
  * segment data: the reference's generate_harmonic_ffdot_data (host code,
    oracle/_ref/libref_u<USELEN>.so) on the whitened spectrum (whitened by
    the reference's deredden);
  * templates: the reference's createSubharmonicInfo (same library), time
    domain;
  * the forward FFTs of segments and templates and the inverse FFTs of the
    convolutions -- cuFFT in the reference (bpd_fft.cu, bpd_search.cu:235,
    :283), which needs a GPU -- in double precision here (numpy), rounded to
    complex64: the exact result the FP32 transforms approximate;
  * convolveSignal, generatePowers and addPowers: the reference's kernel
    source (source/bpd_gpu_kernels.cu) compiled as host C++ and run thread by
    thread over the reference's own launch geometry (bpd_search.cu:249,
    :301, :333) -- oracle/_ref/libref_kernels.so.
Saved per step: the whitened bins the step reads (so a test rebuilds the
exact input without the FFT of the series), the fundamental powers after
generatePowers, the powers after addPowers for counters 1, 3 (and 7) -- the
stage sums of 2, 4 (and 8) harmonics, as test_powers.cu:8-60 records them
-- over a window of columns, and a few rows of the fundamental's
convolution (the quantity test_convolution.cu:7-57 checks).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from gpu_accelsearch_gb300.synth import synth_series  # noqa: E402
from make_golden import DP, FP, IP, fp, reflib, sha  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "reference_planes.npz")
THREADS, KMULT = 128, 30  # bpd_cudacommon.cuh:18-19

# (name, zmax, numharm, uselen, log2 N, steps, column window per step)
CASES = [("c1", 50, 4, 1914, 18, [0, 20], [(0, 512), (1402, 1914)]),
         ("c2", 200, 8, 7734, 22, [5], [(768, 1024)])]
DT = 64e-6
SIGNAL = (0.05, 20000.25, 40.0)


def kernels_lib():
    K = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_kernels.so"))
    U, I, F, D = C.c_uint, C.c_int, C.c_float, C.c_double
    K.ref_launch_convolve.argtypes = [U, U, U, I, I, FP, FP, I, FP]
    K.ref_launch_powers.argtypes = [U, U, U, I, I, I, FP, F, FP]
    K.ref_launch_add_powers.argtypes = [U, U, U, I, I, I, I, I, I, D, FP, F, FP, I]
    return K


def ceil_div(a, b):
    return -(-a // b)


def one_step(R, K, bank, stages, zmax, wspec, startr, uselen):
    nh = 1 << (stages - 1)
    half = uselen // 2
    info = []
    for h in range(nh):
        a = np.zeros(6, np.int32)
        R.ref_bank_info(bank, h, a.ctypes.data_as(IP))
        info.append(a)
    oi = np.zeros(6 * nh, np.int32)
    orhi = np.zeros(nh, np.float64)
    lastr = startr + half - 0.5
    R.ref_step_ffdot(bank, stages, float(startr), lastr, float(-zmax), oi.ctypes.data_as(IP),
                     orhi.ctypes.data_as(DP))
    ff = oi.reshape(nh, 6)  # rlo, numrs, numzs, fftlen, zlo, binoffset
    L = [int(i[4]) for i in info]
    start = np.concatenate([[0], np.cumsum(L)[:-1]]).astype(np.int64)
    total = int(sum(L))
    data = np.zeros(total, np.complex64)
    R.ref_step_data(bank, stages, float(startr), lastr, float(-zmax), fp(wspec.view(np.float32)),
                    wspec.size, fp(data.view(np.float32)))
    # forward FFT of every spread segment (cuFFT stand-in: double, rounded)
    fdata = np.zeros_like(data)
    for h in range(nh):
        s = slice(int(start[h]), int(start[h]) + L[h])
        fdata[s] = np.fft.fft(data[s].astype(np.complex128)).astype(np.complex64)
    # template spectra and the convolution (the reference's kernel)
    conv_off = np.concatenate([[0], np.cumsum([int(i[3]) * L[h] for h, i in enumerate(info)])[:-1]])
    conv = np.zeros(int(sum(int(i[3]) * L[h] for h, i in enumerate(info))), np.complex64)
    for h in range(nh):
        numzs, fftlen = int(info[h][3]), L[h]
        tdom = np.ctypeslib.as_array(R.ref_bank_templates(bank, h), shape=(numzs * fftlen * 2,))
        tdom = tdom.view(np.complex64).reshape(numzs, fftlen)
        kspec = np.fft.fft(tdom.astype(np.complex128), axis=1).astype(np.complex64).ravel()
        seg = np.ascontiguousarray(fdata[int(start[h]): int(start[h]) + fftlen])
        out = np.zeros(numzs * fftlen, np.complex64)
        assert int(ff[h, 3]) == fftlen and int(ff[h, 2]) == numzs
        # grid is an exact multiple of fftlen: the kernel's `> fftlen` bound never lets a thread past it
        assert fftlen % THREADS == 0
        K.ref_launch_convolve(ceil_div(fftlen, THREADS), ceil_div(numzs, KMULT), THREADS, numzs, fftlen,
                              fp(seg.view(np.float32)), fp(kspec.view(np.float32)), fftlen,
                              fp(out.view(np.float32)))
        conv[int(conv_off[h]): int(conv_off[h]) + numzs * fftlen] = out
    # inverse FFTs (cuFFT CUFFT_INVERSE: unnormalised e^{+2 pi i})
    ifft = np.zeros_like(conv)
    for h in range(nh):
        numzs, fftlen = int(info[h][3]), L[h]
        blk = conv[int(conv_off[h]): int(conv_off[h]) + numzs * fftlen].reshape(numzs, fftlen)
        ifft[int(conv_off[h]): int(conv_off[h]) + numzs * fftlen] = (
            np.fft.ifft(blk.astype(np.complex128), axis=1) * fftlen).astype(np.complex64).ravel()
    # generatePowers, then addPowers per counter, keeping the stage sums
    numzs0, numrs0, fftlen0, zlo0 = int(ff[0, 2]), int(ff[0, 1]), L[0], int(ff[0, 4])
    assert numrs0 == uselen
    powers = np.zeros(numzs0 * numrs0, np.float32)
    off0 = int(info[0][5]) * 2
    fund_in = np.ascontiguousarray(ifft[int(conv_off[0]) + off0:])
    K.ref_launch_powers(ceil_div(numrs0, THREADS), ceil_div(numzs0, KMULT), THREADS, numzs0, numrs0, fftlen0,
                        fp(fund_in.view(np.float32)), np.float32(1.0 / (fftlen0 * fftlen0)), fp(powers))
    stages_out = [powers.reshape(numzs0, numrs0).copy()]
    for c in range(1, nh):
        frac = float(info[c][0]) / float(info[c][1])
        off = int(info[c][5]) * 2
        sub = np.ascontiguousarray(ifft[int(conv_off[c]) + off:])
        K.ref_launch_add_powers(ceil_div(numrs0, THREADS), ceil_div(numzs0, KMULT), THREADS, numzs0, numrs0,
                                L[c], zlo0, int(ff[c, 4]), int(ff[c, 0]), frac, fp(sub.view(np.float32)),
                                np.float32(1.0 / (L[c] * L[c])), fp(powers), int(startr))
        if ((c + 1) & c) == 0:
            stages_out.append(powers.reshape(numzs0, numrs0).copy())
    # the whitened bins each harmonic's segment reads (lobin = rlo - binoffset,
    # fftlen / 2 of them), with a margin
    ranges = []
    for h in range(nh):
        lo = int(ff[h, 0]) - int(ff[h, 5]) - 8
        hi = lo + L[h] // 2 + 16
        ranges.append((max(lo, 0), min(hi, wspec.size)))
    conv0 = conv[: int(info[0][3]) * L[0]].reshape(int(info[0][3]), L[0])
    return stages_out, ranges, conv0


def main():
    K = kernels_lib()
    out = {}
    for name, zmax, numharm, uselen, nlog2, steps, windows in CASES:
        R = reflib(uselen)
        stages = int(np.log2(numharm)) + 1
        bank = R.ref_create_bank(stages, zmax)
        n = 1 << nlog2
        x = synth_series(n, seed=1000 + nlog2, signals=[SIGNAL])
        spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)
        numbins = n // 2
        w = spec[:numbins].copy()
        R.ref_deredden(fp(w.view(np.float32)), numbins)
        rlo = int(np.floor(1.0 * float(np.float32(n) * np.float32(DT))))
        out[f"{name}_meta"] = np.array([zmax, numharm, uselen, n, numbins, rlo], np.int64)
        out[f"{name}_whitened_sha"] = np.frombuffer(bytes.fromhex(sha(w)), np.uint8)
        for k, (c0, c1) in zip(steps, windows):
            startr = rlo + k * (uselen // 2)
            st, ranges, conv0 = one_step(R, K, bank, stages, zmax, w, startr, uselen)
            key = f"{name}_s{k}"
            out[key + "_startr"] = np.array([startr], np.int64)
            out[key + "_window"] = np.array([c0, c1], np.int64)
            out[key + "_stages"] = np.stack([a[:, c0:c1] for a in st]).astype(np.float32)
            out[key + "_ranges"] = np.array(ranges, np.int64)
            out[key + "_bins"] = np.concatenate([w[a:b] for a, b in ranges]).astype(np.complex64)
            if name == "c1" and k == steps[-1]:
                rows = np.array([0, conv0.shape[0] // 2, conv0.shape[0] - 1], np.int64)
                out[key + "_conv_rows"] = rows
                out[key + "_conv"] = conv0[rows].astype(np.complex64)
            print(name, "step", k, "startr", startr, "stages", len(st), "peak",
                  float(max(a[:, c0:c1].max() for a in st)))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
