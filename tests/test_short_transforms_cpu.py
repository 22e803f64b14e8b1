"""Short transforms (accel_config.short_transforms), on the CPU in FP64.

The reference transforms each harmonic's segment at the power of two above
its data (bpd_subharmonics.cu:60-67) and keeps the plane columns
[2 hw0, 2 hw0 + numrs).  Any even length L' >= 2 numdata gives the same
kept columns: they are a linear correlation of the first numdata bins with
templates of halfwidth <= hw0, and the circular wrap of the shorter
transform only reaches the columns below 2 hw0.  This file checks that claim
with the oracle's own segment and template builders at the lengths the
library picks (the smallest R * 2^k, R in {5, 6, 7}, 64 <= 2^k <= 512,
holding numdata), and checks the kernels' decomposition of such a transform
-- R transforms of 2^k points over the decimated order, then one radix-R
pass -- against numpy's FFT.
"""
import numpy as np
import pytest

from oracle import oracle as O


def short_half_length(M, numdata):
    """The library's choice (api.cu short_half_length): the smallest R * N2
    >= numdata below the power of two M, else M."""
    best = M
    for R in (5, 6, 7):
        n2 = 64
        while n2 <= 512:
            if numdata <= R * n2 < best:
                best = R * n2
            n2 *= 2
    return best


def numdata_max(p, q, U, hw0):
    nd = 0
    for s in range(4 * q):
        startr = 1000000 + s
        rlo, rhi, _, _ = O.step_ffdot(p, q, 200, U, startr, startr + U / 2 - 0.5)
        nd = max(nd, int(np.ceil(rhi)) - rlo + 2 * hw0 + 1)
    return nd


@pytest.mark.parametrize("L", [4096, 8192])
def test_short_lengths_keep_the_same_powers(L):
    rng = np.random.default_rng(L)
    spec = (rng.standard_normal(1 << 19) + 1j * rng.standard_normal(1 << 19)).astype(np.complex64)
    U = L - 2 - 4 * O.z_halfwidth(200)
    geom = O.bank_geometry(200, 8, U)
    shortened = 0
    for p, q, zmax_h, numzs, Lh, hw0, zlo in (map(int, r) for r in geom[1:]):
        M = Lh // 2
        Ms = short_half_length(M, numdata_max(p, q, U, hw0))
        if Ms == M:
            continue
        shortened += 1
        assert Ms % 2 == 0 and Ms < M
        for startr in (1000, 54321):
            rlo, rhi, _, numrs = O.step_ffdot(p, q, 200, U, startr, startr + U / 2 - 0.5)
            seg = O.segment_data(spec, rlo, rhi, hw0, Lh).astype(np.complex128)
            for z in (-zmax_h, 0, zmax_h):
                y = np.fft.ifft(np.fft.fft(seg) * np.fft.fft(O.wrapped_template(Lh, z).astype(np.complex128)))
                ys = np.fft.ifft(np.fft.fft(seg[: 2 * Ms]) *
                                 np.fft.fft(O.wrapped_template(2 * Ms, z).astype(np.complex128)))
                # ifft(fft(a) fft(b)) is the circular convolution itself at either length
                a = np.abs(y[2 * hw0: 2 * hw0 + numrs]) ** 2
                b = np.abs(ys[2 * hw0: 2 * hw0 + numrs]) ** 2
                assert np.max(np.abs(a - b)) <= 1e-9 * np.max(a), (p, q, z)
    # at zmax 200 / 8 harmonics: 1/4, 3/4, 1/8, 3/8, 5/8, 7/8
    assert shortened == 6


@pytest.mark.parametrize("R,N2", [(5, 64), (6, 256), (7, 128), (7, 512)])
@pytest.mark.parametrize("direction", [-1, 1])
def test_decimated_radix_r_decomposition(R, N2, direction):
    M = R * N2
    rng = np.random.default_rng(M + direction)
    x = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    # storage in decimated order: position g N2 + n holds point R n + g
    dec = np.empty(M, complex)
    for k in range(M):
        dec[(k % R) * N2 + k // R] = x[k]
    # R transforms of N2 points, one per group g
    Y = np.array([np.fft.fft(dec[g * N2:(g + 1) * N2]) if direction < 0 else
                  np.fft.ifft(dec[g * N2:(g + 1) * N2]) * N2 for g in range(R)])
    # radix-R pass: X[b + N2 k1] = sum_g W_R^(g k1) W_M^(g b) Y_g[b]
    X = np.empty(M, complex)
    b = np.arange(N2)
    for k1 in range(R):
        acc = np.zeros(N2, complex)
        for g in range(R):
            acc += np.exp(direction * 2j * np.pi * g * k1 / R) * np.exp(direction * 2j * np.pi * g * b / M) * Y[g]
        X[b + N2 * k1] = acc
    want = np.fft.fft(x) if direction < 0 else np.fft.ifft(x) * M
    assert np.allclose(X, want, rtol=0, atol=1e-9 * np.abs(want).max())
