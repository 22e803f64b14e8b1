"""GPU path against the FP64 oracle at the bench's geometry and its
neighbours, through the C ABI (the main parity file runs zmax 50, 4
harmonics, L 2048): zmax 200 with 8 harmonics at L = 4096, 8192 (the bench)
and 16384, 16 harmonics at zmax 100, and the serving banks zmax 300, 100
and 50 with 8 harmonics at L = 8192.  Between them they run every
plane-kernel size class (M = 512 .. 8192) and the 8- and 16-harmonic sums.

Tolerances as in test_gpu_parity.py: power planes max |P - P64| /
max(P64, 1) < 1e-4; candidates identical outside a +-1e-4 relative band
around each stage's cut.
"""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_P = 1e-4
# the serving banks at the serving segment length: zmax 300, 100 and 50
# with 8 harmonics at L = 8192
GEOMS = [(200, 8, 8192), (200, 8, 4096), (200, 8, 16384), (100, 16, 8192),
         (300, 8, 8192), (100, 8, 8192), (50, 8, 8192)]
RLO = 16
SIG_STEP = 10


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.float32).copy()).cuda()


# every geometry with the reference's power-of-two transforms and with the
# short transforms (R * 2^k points, R = 5, 6, 7: the 3/4, 5/8, 7/8, 1/4, 3/8
# and 1/8 harmonics at zmax 200)
@pytest.fixture(scope="module", params=[g + (sh,) for sh in (False, True) for g in GEOMS],
                ids=lambda g: "z%d_h%d_L%d" % g[:3] + ("_short" if g[3] else ""))
def G(request):
    from gpu_accelsearch_gb300.search import AccelSearch
    zmax, nh, L, short = request.param
    s = AccelSearch(zmax=zmax, numharm=nh, fftlen=L, short_transforms=short)
    if short:  # some harmonic really runs a short transform
        assert any(h.fftlen & (h.fftlen - 1) for h in s.harmonics), s.harmonics
    U = s.uselen
    n = 1 << 20
    # one accelerated signal in the middle of step SIG_STEP's fundamental range
    r0 = RLO + SIG_STEP * (U // 2) + U // 4 + 0.25
    x = synth_series(n, seed=2000 + L + nh, signals=[(0.04, r0, 30.0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
    w = O.deredden(spec)
    o = O.Oracle(zmax, nh, U)
    yield {"s": s, "o": o, "w": w, "zmax": zmax, "r0": r0}
    o.close()
    s.close()


def test_power_planes_every_harmonic(G):
    s, o, w = G["s"], G["o"], G["w"]
    U = s.uselen
    startr = [RLO + SIG_STEP * (U // 2), RLO + (SIG_STEP + 1) * (U // 2)]
    d = dev(w)
    dh = torch.zeros(len(startr) * s.dhalf_stride * 2, dtype=torch.float32, device="cuda")
    pl = torch.zeros(len(startr) * s.plane_stride, dtype=torch.float32, device="cuda")
    s.prepare_segments(d.data_ptr(), w.size, startr, dh.data_ptr())
    s.power_planes(dh.data_ptr(), len(startr), pl.data_ptr())
    P = pl.cpu().numpy().reshape(len(startr), s.plane_stride)
    peak = 0.0
    for si, s0 in enumerate(startr):
        for h in range(len(s.harmonics)):
            p64 = o.harmonic_plane(w, float(s0), h)
            nz, nr = p64.shape
            g = P[si, s.plane_off[h]: s.plane_off[h] + nz * s.plane_row[h]].reshape(
                nz, s.plane_row[h])[:, :nr]
            err = (np.abs(g - p64) / np.maximum(p64, 1.0)).max()
            assert err < TOL_P, (si, h, err)
            peak = max(peak, float(p64.max()))
    assert peak > 50.0  # the injected signal is in these planes


def _keys(a, rlo, half, zlo0):
    if "ridx" in a.dtype.names:
        return {(int(c["step"]), int(c["ridx"]), int(c["zidx"]), int(c["numharm"])) for c in a}
    return {(int(c["step"]), int(round(2 * (c["r"] - (rlo + c["step"] * half)))),
             int(round((c["z"] - zlo0) / 2)), int(c["numharm"])) for c in a}


def test_candidates_match_oracle(G):
    # ~3.5 sigma cuts: thousands of candidates through the tiled sum and the
    # compaction; steps 8..12 around the signal
    s, o, w = G["s"], G["o"], G["w"]
    U = s.uselen
    cuts = np.array([O.power_cut(3.5, 1 << k) for k in range(s.nstages)])
    s.set_power_cuts(cuts.astype(np.float32))
    try:
        d = dev(w)
        s.search_spectra([d.data_ptr()], [w.size], [RLO])
        gpu = s.candidates()
    finally:
        s.set_power_cuts([O.power_cut(6.0, 1 << k) for k in range(s.nstages)])
    step0, nsteps = SIG_STEP - 2, 5
    gpu = gpu[(gpu["step"] >= step0) & (gpu["step"] < step0 + nsteps)]
    c32 = cuts.astype(np.float32).astype(np.float64)
    lo, _, _ = o.run_steps(w, RLO, step0, nsteps, powcut=c32 * (1 - TOL_P), cap=1 << 22)
    hi, _, _ = o.run_steps(w, RLO, step0, nsteps, powcut=c32 * (1 + TOL_P), cap=1 << 22)
    g = _keys(gpu, RLO, U // 2, -G["zmax"])
    assert len(g) > 1000
    assert _keys(hi, 0, 0, 0) <= g <= _keys(lo, 0, 0, 0)
    # the strongest single-harmonic candidate is the injected signal: r0 + z/2
    # at the middle of the observation, z = 30 (summed stages also peak where a
    # sub-harmonic lands on it, e.g. at 8/7 of its frequency)
    one = gpu[gpu["numharm"] == 1]
    best = one[np.argmax(one["power"])]
    assert abs(best["r"] - (G["r0"] + 15.0)) <= 1.0 and abs(best["z"] - 30) <= 4
