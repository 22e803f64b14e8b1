"""The GPU path against golden planes from the reference's own code
(tests/golden/reference_planes.npz, written by
tests/golden/make_plane_golden.py): the reference's host segment
preparation and templates, its three kernels' source (convolveSignal,
generatePowers, addPowers) run over its own launch geometry, and
double-precision transforms in place of cuFFT.  Checked, per stored step
of the small configuration (zmax 50, 4 harmonics, L 2048: steps 0 and 20)
and of the single-trial configuration (zmax 200, 8 harmonics, L 8192: the
step holding the signal):
  * the fused path's fundamental powers and harmonic stage sums -- the
    powers after the reference's addPowers counters 1, 3 and 7 -- within
    |P - Pref| / max(Pref, 1) < 1e-4;
  * the drop-in layer's perform_convolution (test_convolution.cu's quantity)
    within 1e-5 of the largest value, and its generate_fundamental_powers
    and perform_harmonic_summing within 1e-4, driven through the
    reference's step sequence.
"""
import ctypes as C

import numpy as np
import pytest

import golden_planes as GP

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
TOL_P = 1e-4


@pytest.fixture(scope="module")
def g():
    return GP.load()


def fundamental_fftlen(zmax, uselen):
    from oracle import oracle as O
    return O.fft_length(1, 1, zmax, uselen)


@pytest.mark.parametrize("which", range(3))
def test_fused_path_equals_reference_kernels(g, which):
    from gpu_accelsearch_gb300.search import AccelSearch
    case, step, zmax, numharm, uselen, numbins, startr, (c0, c1), ref = GP.cases(g)[which]
    w = GP.spectrum(g, case, step, numbins)
    with AccelSearch(zmax=zmax, numharm=numharm, fftlen=fundamental_fftlen(zmax, uselen)) as s:
        assert s.uselen == uselen
        d = torch.from_numpy(w.view(np.float32).copy()).cuda()
        dh = torch.zeros(s.dhalf_stride * 2, dtype=torch.float32, device="cuda")
        pl = torch.zeros(s.plane_stride, dtype=torch.float32, device="cuda")
        s.prepare_segments(d.data_ptr(), numbins, [startr], dh.data_ptr())
        s.power_planes(dh.data_ptr(), 1, pl.data_ptr())
        nz = s.harmonics[0].numzs
        st = torch.zeros(s.nstages * nz * uselen, dtype=torch.float32, device="cuda")
        s.sum_harmonics(pl.data_ptr(), [startr], st.data_ptr())
        got = st.cpu().numpy().reshape(s.nstages, nz, uselen)[:, :, c0:c1]
        fund = pl.cpu().numpy()[s.plane_off[0]: s.plane_off[0] + nz * s.plane_row[0]]
        fund = fund.reshape(nz, s.plane_row[0])[:, c0:c1]
    assert got.shape == ref.shape
    err = (np.abs(got - ref) / np.maximum(ref, 1.0)).max(axis=(1, 2))
    assert (err < TOL_P).all(), (case, step, err)
    assert (np.abs(fund - ref[0]) / np.maximum(ref[0], 1.0)).max() < TOL_P


def test_drop_in_stages_equal_reference_kernels(g):
    from gpu_accelsearch_gb300 import compat as CP
    L = CP.lib()
    case, step, zmax, numharm, uselen, numbins, startr, (c0, c1), ref = [
        c for c in GP.cases(g) if c[0] == "c1"][-1]
    key = f"{case}_s{step}"
    conv_rows, conv_ref = g[key + "_conv_rows"], g[key + "_conv"]
    w = GP.spectrum(g, case, step, numbins)
    stages = int(np.log2(numharm)) + 1
    L.accel_compat_set_uselen(uselen)
    shi = L.createSubharmonicInfo(stages, zmax)
    CP.check()
    nh = L.getTotalHarmonics(stages)
    starts = (C.c_long * nh)()
    conv_idx = (C.c_long * nh)()
    tot = tot_conv = 0
    for h in range(nh):
        starts[h], conv_idx[h] = tot, tot_conv
        tot += shi[h].kernelFFTLength
        tot_conv += shi[h].kernelFFTLength * shi[h].totalKernelsTemplates
    L.initialize_cuda_plans(nh, shi)
    CP.check()
    try:
        d_data = torch.zeros(2 * tot, dtype=torch.float32, device="cuda")
        d_fft = torch.zeros_like(d_data)
        d_conv = torch.zeros(2 * tot_conv, dtype=torch.float32, device="cuda")
        d_ifft = torch.zeros_like(d_conv)
        nz0, L0 = shi[0].totalKernelsTemplates, shi[0].kernelFFTLength
        d_pow = torch.zeros(nz0 * uselen, dtype=torch.float32, device="cuda")
        host = np.zeros(tot, np.complex64)
        fi = (CP.FfdotInfo * nh)()
        bo = (C.c_ushort * nh)()
        L.generate_harmonics_ffdot(nh, stages, shi, startr, startr + uselen // 2 - 0.5, -zmax, fi, bo)
        L.generate_harmonic_ffdot_data(nh, tot, fi, bo, starts, w.ctypes.data, w.size, 0, host.ctypes.data)
        d_data.copy_(torch.from_numpy(host.view(np.float32)))
        L.perform_fft_harmonics(nh, d_data.data_ptr(), starts, d_fft.data_ptr())
        L.perform_convolution(nh, d_fft.data_ptr(), fi, shi, starts, d_conv.data_ptr(), conv_idx)
        torch.cuda.synchronize()
        CP.check()
        conv = d_conv.cpu().numpy().view(np.complex64)[: nz0 * L0].reshape(nz0, L0)[conv_rows]
        assert np.abs(conv - conv_ref).max() / np.abs(conv_ref).max() < 1e-5
        L.perform_inversefft(nh, d_conv.data_ptr(), conv_idx, d_ifft.data_ptr())
        L.generate_fundamental_powers(nh, d_ifft.data_ptr(), conv_idx, fi, shi, d_pow.data_ptr())
        torch.cuda.synchronize()
        CP.check()
        p0 = d_pow.cpu().numpy().reshape(nz0, uselen)[:, c0:c1]
        assert (np.abs(p0 - ref[0]) / np.maximum(ref[0], 1.0)).max() < TOL_P
        L.perform_harmonic_summing(nh, d_ifft.data_ptr(), conv_idx, fi, shi, d_pow.data_ptr(), int(startr),
                                   None, None, 0)
        torch.cuda.synchronize()
        CP.check()
        pn = d_pow.cpu().numpy().reshape(nz0, uselen)[:, c0:c1]
        assert (np.abs(pn - ref[-1]) / np.maximum(ref[-1], 1.0)).max() < TOL_P
    finally:
        L.free_cuda_plans(nh)
        L.freeSubharmonicInfo(shi, nh)
        L.accel_compat_set_uselen(32000)
