"""The exact_rsqrt option through the C ABI: whitening and the per-segment
normalisation use IEEE 1/sqrt instead of the reference's magic-constant
rsqrt.  Checked against the oracle switched to the same arithmetic:
  * whitening bit-identical;
  * power planes within |P - P64| / max(P64, 1) < 1e-4;
  * candidates identical outside the +-1e-4 band around each cut;
and the option measurably changes the planes (the magic rsqrt is ~1e-3
off), so the flag reaches the kernels.
"""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_red_spectrum, synth_series
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_P = 1e-4


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.float32).copy()).cuda()


@pytest.fixture
def exact_oracle():
    O.set_exact_rsqrt(True)
    yield
    O.set_exact_rsqrt(False)


@pytest.fixture(scope="module")
def trial():
    n = 1 << 18
    x = synth_series(n, seed=1018, signals=[(0.05, 20000.25, 40.0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
    return {"spec": spec}


@pytest.mark.parametrize("numbins", [1 << 17, 12345])
def test_whitening_bit_exact(numbins, exact_oracle):
    from gpu_accelsearch_gb300.search import AccelSearch
    spec = synth_red_spectrum(numbins, seed=numbins)
    with AccelSearch(zmax=50, numharm=4, fftlen=2048, exact_rsqrt=True) as s:
        d = dev(spec)
        s.whiten(d.data_ptr(), numbins)
        s.synchronize()
        got = d.cpu().numpy().view(np.complex64)
    want = O.deredden(spec)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _planes(s, w, startr):
    d = dev(w)
    dh = torch.zeros(len(startr) * s.dhalf_stride * 2, dtype=torch.float32, device="cuda")
    pl = torch.zeros(len(startr) * s.plane_stride, dtype=torch.float32, device="cuda")
    s.prepare_segments(d.data_ptr(), w.size, startr, dh.data_ptr())
    s.power_planes(dh.data_ptr(), len(startr), pl.data_ptr())
    return pl.cpu().numpy().reshape(len(startr), s.plane_stride)


def test_planes_and_candidates(trial, exact_oracle):
    from gpu_accelsearch_gb300.search import AccelSearch
    w = O.deredden(trial["spec"])
    startr = [16 + 957 * 20]
    o = O.Oracle(50, 4, 1914)
    try:
        with AccelSearch(zmax=50, numharm=4, fftlen=2048, exact_rsqrt=True) as s, \
                AccelSearch(zmax=50, numharm=4, fftlen=2048) as m:
            P = _planes(s, w, startr)[0]
            Pm = _planes(m, w, startr)[0]
            worst, moved = 0.0, 0.0
            for h, hi in enumerate(s.harmonics):
                p64 = o.harmonic_plane(w, float(startr[0]), h)
                nz, nr = p64.shape
                cut = lambda a: a[s.plane_off[h]: s.plane_off[h] + nz * s.plane_row[h]].reshape(
                    nz, s.plane_row[h])[:, :nr]
                g, gm = cut(P), cut(Pm)
                worst = max(worst, (np.abs(g - p64) / np.maximum(p64, 1.0)).max())
                moved = max(moved, (np.abs(g - gm) / np.maximum(g, 1.0)).max())
            assert worst < TOL_P, worst
            assert moved > 3e-4, moved
            d = dev(w)
            s.search_spectra([d.data_ptr()], [w.size], [16])
            gpu = s.candidates()
            cuts = s.power_cuts().astype(np.float64)
            steps = 24
            gpu = gpu[gpu["step"] < steps]
            lo, _, _ = o.run_steps(w, 16, 0, steps, powcut=cuts * (1 - TOL_P), cap=1 << 22)
            hi, _, _ = o.run_steps(w, 16, 0, steps, powcut=cuts * (1 + TOL_P), cap=1 << 22)
            half = s.uselen // 2
    finally:
        o.close()
    g = {(int(c["step"]), int(round(2 * (c["r"] - (16 + c["step"] * half)))),
          int(round((c["z"] + 50) / 2)), int(c["numharm"])) for c in gpu}
    k = lambda a: {(int(c["step"]), int(c["ridx"]), int(c["zidx"]), int(c["numharm"])) for c in a}
    assert len(g) > 0
    assert k(hi) <= g <= k(lo)
