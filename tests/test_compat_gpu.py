"""The drop-in layer (include/bpd_compat.h) on the GPU, driven with the
reference's own per-step call sequence (AccelSearch.cu:209-245), against
the FP64 oracle.  Tolerances as in test_gpu_parity: powers
|P - P64| / max(P64, 1) < 1e-4, whitening bit-exact, FFTs 1e-5 of max."""
import ctypes as C

import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_red_spectrum, synth_series
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
TOL_P = 1e-4


def cudart():
    for name in ("/usr/local/cuda/lib64/libcudart.so", "libcudart.so", "libcudart.so.13"):
        try:
            lib = C.CDLL(name)
            lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            lib.cudaFree.argtypes = [C.c_void_p]
            return lib
        except OSError:
            continue
    pytest.skip("libcudart not found")


def dev_to_host(ptr, n, dtype):
    out = np.empty(n, dtype)
    assert cudart().cudaMemcpy(out.ctypes.data, ptr, out.nbytes, 2) == 0
    return out


@pytest.fixture(scope="module")
def L():
    from gpu_accelsearch_gb300 import compat as CP
    return CP.lib()


def test_reference_step_sequence(L):
    from gpu_accelsearch_gb300 import compat as CP
    zmax, stages, U, n = 50, 3, 1914, 1 << 18
    L.accel_compat_set_uselen(U)
    shi = L.createSubharmonicInfo(stages, zmax)
    CP.check()
    nh = L.getTotalHarmonics(stages)
    # the template spectra left in kernels_data
    for h in range(nh):
        s = shi[h]
        k = dev_to_host(s.kernels_data, s.totalKernelsTemplates * s.kernelFFTLength, np.complex64)
        k = k.reshape(s.totalKernelsTemplates, s.kernelFFTLength)
        k64 = np.stack([O.fft64(O.wrapped_template(s.kernelFFTLength, -s.zmax + 2 * j))
                        for j in range(s.totalKernelsTemplates)])
        assert np.abs(k - k64).max() / np.abs(k64).max() < 2e-6
    x = synth_series(n, seed=1018, signals=[(0.05, 20000.25, 40.0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)
    w = O.deredden(spec[: n // 2])
    starts = (C.c_long * nh)()
    conv_idx = (C.c_long * nh)()
    tot = tot_conv = 0
    for h in range(nh):
        starts[h], conv_idx[h] = tot, tot_conv
        tot += shi[h].kernelFFTLength
        tot_conv += shi[h].kernelFFTLength * shi[h].totalKernelsTemplates
    L.initialize_cuda_plans(nh, shi)
    CP.check()
    d_data = torch.zeros(2 * tot, dtype=torch.float32, device="cuda")
    d_fft = torch.zeros_like(d_data)
    d_conv = torch.zeros(2 * tot_conv, dtype=torch.float32, device="cuda")
    d_ifft = torch.zeros_like(d_conv)
    nz0 = shi[0].totalKernelsTemplates
    d_pow = torch.zeros(nz0 * U, dtype=torch.float32, device="cuda")
    host = np.zeros(tot, np.complex64)
    fi = (CP.FfdotInfo * nh)()
    bo = (C.c_ushort * nh)()
    orc = O.Oracle(zmax, nh, U)
    cuts = [O.power_cut(6.0, 1 << s) for s in range(orc.nstages)]
    for step in (0, 20, 135):
        startr = 16 + step * (U // 2)
        L.generate_harmonics_ffdot(nh, stages, shi, startr, startr + U // 2 - 0.5, -zmax, fi, bo)
        L.generate_harmonic_ffdot_data(nh, tot, fi, bo, starts, w.ctypes.data, w.size, 0,
                                       host.ctypes.data)
        d_data.copy_(torch.from_numpy(host.view(np.float32)))
        L.perform_fft_harmonics(nh, d_data.data_ptr(), starts, d_fft.data_ptr())
        L.perform_convolution(nh, d_fft.data_ptr(), fi, shi, starts, d_conv.data_ptr(), conv_idx)
        L.perform_inversefft(nh, d_conv.data_ptr(), conv_idx, d_ifft.data_ptr())
        L.generate_fundamental_powers(nh, d_ifft.data_ptr(), conv_idx, fi, shi, d_pow.data_ptr())
        torch.cuda.synchronize()
        CP.check()
        _, planes, _ = orc.run_steps(w, 16, step, 1, want_planes=True)
        p1 = d_pow.cpu().numpy().reshape(nz0, U)
        assert (np.abs(p1 - planes[0, 0]) / np.maximum(planes[0, 0], 1.0)).max() < TOL_P
        L.perform_harmonic_summing(nh, d_ifft.data_ptr(), conv_idx, fi, shi, d_pow.data_ptr(),
                                   int(startr), None, None, 0)
        torch.cuda.synchronize()
        CP.check()
        pn = d_pow.cpu().numpy().reshape(nz0, U)
        last = planes[0, -1]
        assert (np.abs(pn - last) / np.maximum(last, 1.0)).max() < TOL_P
        # candidates of the summed plane
        nc = C.c_long(0)
        cptr = L.search_ffdot_powers_n(fi, nh, cuts[-1], 1, C.byref(nc))
        CP.check()
        got = {(round(2 * (cptr[k].r - startr)), round((cptr[k].z + zmax) / 2))
               for k in range(nc.value)}
        lo = {(i, z) for z, i in zip(*np.nonzero(last > cuts[-1] * (1 - TOL_P)))}
        hi = {(i, z) for z, i in zip(*np.nonzero(last > cuts[-1] * (1 + TOL_P)))}
        assert hi <= got <= lo
    L.free_cuda_plans(nh)
    L.freeSubharmonicInfo(shi, nh)
    L.accel_compat_set_uselen(32000)


def test_reference_kernel_launchers(L):
    # convolveSignal / generatePowers / addPowers (bpd_gpu_kernels.cuh:15-17)
    # called as the reference's stage functions call them give exactly the
    # stage functions' outputs
    from gpu_accelsearch_gb300 import compat as CP
    zmax, stages, U, n = 50, 3, 1914, 1 << 18
    L.accel_compat_set_uselen(U)
    shi = L.createSubharmonicInfo(stages, zmax)
    nh = L.getTotalHarmonics(stages)
    x = synth_series(n, seed=1019, signals=[(0.05, 20000.25, 40.0)])
    w = O.deredden(np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2])
    starts = (C.c_long * nh)()
    conv_idx = (C.c_long * nh)()
    tot = tot_conv = 0
    for h in range(nh):
        starts[h], conv_idx[h] = tot, tot_conv
        tot += shi[h].kernelFFTLength
        tot_conv += shi[h].kernelFFTLength * shi[h].totalKernelsTemplates
    L.initialize_cuda_plans(nh, shi)
    d_data = torch.zeros(2 * tot, dtype=torch.float32, device="cuda")
    d_fft = torch.zeros_like(d_data)
    d_conv, d_conv2 = (torch.zeros(2 * tot_conv, dtype=torch.float32, device="cuda") for _ in range(2))
    d_ifft = torch.zeros_like(d_conv)
    nz0 = shi[0].totalKernelsTemplates
    d_pow, d_pow2 = (torch.zeros(nz0 * U, dtype=torch.float32, device="cuda") for _ in range(2))
    host = np.zeros(tot, np.complex64)
    fi = (CP.FfdotInfo * nh)()
    bo = (C.c_ushort * nh)()
    startr = 16 + 20 * (U // 2)
    L.generate_harmonics_ffdot(nh, stages, shi, startr, startr + U // 2 - 0.5, -zmax, fi, bo)
    L.generate_harmonic_ffdot_data(nh, tot, fi, bo, starts, w.ctypes.data, w.size, 0, host.ctypes.data)
    d_data.copy_(torch.from_numpy(host.view(np.float32)))
    L.perform_fft_harmonics(nh, d_data.data_ptr(), starts, d_fft.data_ptr())
    L.perform_convolution(nh, d_fft.data_ptr(), fi, shi, starts, d_conv.data_ptr(), conv_idx)
    for h in range(nh):
        L.convolveSignal(shi[h].totalKernelsTemplates, shi[h].kernelFFTLength,
                         d_fft.data_ptr() + 8 * starts[h], shi[h].kernels_data, shi[h].kernelFFTLength,
                         d_conv2.data_ptr() + 8 * conv_idx[h])
        CP.check()
    torch.cuda.synchronize()
    assert torch.equal(d_conv.view(torch.int32), d_conv2.view(torch.int32))
    L.perform_inversefft(nh, d_conv.data_ptr(), conv_idx, d_ifft.data_ptr())
    L.generate_fundamental_powers(nh, d_ifft.data_ptr(), conv_idx, fi, shi, d_pow.data_ptr())
    off0 = 2 * shi[0].kernelHalfWidth[0]
    L.generatePowers(fi[0].numzs, fi[0].numrs, fi[0].fftlen, d_ifft.data_ptr() + 8 * (conv_idx[0] + off0),
                     float(np.float32(1.0 / (fi[0].fftlen * fi[0].fftlen))), d_pow2.data_ptr())
    CP.check()
    torch.cuda.synchronize()
    assert torch.equal(d_pow.view(torch.int32), d_pow2.view(torch.int32))
    L.perform_harmonic_summing(nh, d_ifft.data_ptr(), conv_idx, fi, shi, d_pow.data_ptr(), int(startr),
                               None, None, 0)
    for h in range(1, nh):
        off = 2 * shi[h].kernelHalfWidth[0]
        L.addPowers(fi[0].numzs, fi[0].numrs, fi[h].fftlen, fi[0].zlo, fi[h].zlo, fi[h].rlo,
                    fi[h].currentHarmonic / fi[h].maxHarmonic, d_ifft.data_ptr() + 8 * (conv_idx[h] + off),
                    float(np.float32(1.0 / (fi[h].fftlen * fi[h].fftlen))), d_pow2.data_ptr(), int(startr))
        CP.check()
    torch.cuda.synchronize()
    assert torch.equal(d_pow.view(torch.int32), d_pow2.view(torch.int32))
    L.addPowers(1, 1, 2048, 0, 0, 0, 1.0 / 3.0, d_ifft.data_ptr(), 1.0, d_pow2.data_ptr(), 0)
    assert L.accel_compat_status() == -1  # not p / 2^k
    L.free_cuda_plans(nh)
    L.freeSubharmonicInfo(shi, nh)
    L.accel_compat_set_uselen(32000)


@pytest.mark.parametrize("length,batch", [(2048, 3), (16384, 2), (32768, 1)])
def test_c2c_transforms(L, length, batch):
    rng = np.random.default_rng(length)
    x = (rng.standard_normal((batch, length)) + 1j * rng.standard_normal((batch, length))).astype(np.complex64)
    d = torch.from_numpy(x.view(np.float32).reshape(-1).copy()).cuda()
    for fn, ref in ((L.complexToComplexFFT, np.fft.fft),
                    (L.inverseComplexToComplexFFT, lambda a, axis: np.fft.ifft(a, axis=axis) * a.shape[axis])):
        out = C.c_void_p()
        assert fn(d.data_ptr(), length, C.byref(out), batch) == length, L.accel_last_error()
        y = dev_to_host(out.value, batch * length, np.complex64).reshape(batch, length)
        cudart().cudaFree(out.value)
        want = ref(x.astype(np.complex128), axis=1)
        assert np.abs(y - want).max() / np.abs(want).max() < 1e-5


def test_deredden_host_array(L):
    spec = synth_red_spectrum(1 << 16, seed=3)
    got = spec.copy()
    L.deredden(got.ctypes.data, got.size)
    assert L.accel_compat_status() == 0
    assert np.array_equal(got.view(np.uint32), O.deredden(spec).view(np.uint32))


def test_real_to_complex(L):
    x = synth_series(1 << 16, seed=9)
    out = C.c_void_p()
    nout = L.realToComplexFFT(x.ctypes.data_as(C.POINTER(C.c_float)), x.size, C.byref(out), 1)
    assert nout == x.size // 2 + 1
    y = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_float)), shape=(2 * nout,)).copy()
    C.CDLL(None).free(out)
    want = np.fft.rfft(x.astype(np.float64))
    assert np.abs(y.view(np.complex64) - want).max() / np.abs(want).max() < 1e-5
