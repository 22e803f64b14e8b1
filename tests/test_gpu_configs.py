"""The small plain configuration with its own whitening (1000-bin blocks)
and the serving configuration's largest bank (zmax 300), through the C ABI,
against the FP64 oracle on every overlap-save step.

Tolerances as in test_gpu_parity.py: whitening bit-identical; candidates
identical outside a +-1e-4 relative band around each stage's cut.
"""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series
from oracle import oracle as O
from parity_keys import keys, oracle_bounds

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DT = 64e-6


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.float32).copy()).cuda()


def host_c64(t):
    return t.cpu().numpy().view(np.complex64)


def test_small_config_with_1000_bin_whitening():
    # N = 2^18, one accelerated signal (A 0.05, r0 20000.25, z 40), whitening
    # by constant 1000-bin blocks (deredden with initial and maximum block
    # length 1000), zmax 50, 4 harmonics, 2048-point segments, sigma 6
    from gpu_accelsearch_gb300.search import AccelSearch, first_bin
    n = 1 << 18
    x = synth_series(n, seed=1018, signals=[(0.05, 20000.25, 40.0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
    rlo = first_bin(n, DT)
    with AccelSearch(zmax=50, numharm=4, fftlen=2048, whiten_initbuf=1000, whiten_maxbuf=1000) as s:
        d = dev(spec)
        s.whiten(d.data_ptr(), spec.size)
        s.synchronize()
        w = host_c64(d)
        want = O.deredden(spec, 1000, 1000)
        assert np.array_equal(w.view(np.uint32), want.view(np.uint32))
        s.search_spectra([d.data_ptr()], [w.size], [rlo])
        gpu = s.candidates()
        cuts = s.power_cuts().astype(np.float64)
        nsteps = s.step_count(n, DT)
        half = s.uselen // 2
        # the whole path from the series (cuFFT R2C, 1000-bin whitening) equals
        # the stage calls it is made of
        xd = torch.from_numpy(x).cuda()
        sp = torch.zeros((n // 2 + 1) * 2, dtype=torch.float32, device="cuda")
        s.rfft(xd.data_ptr(), n, sp.data_ptr())
        s.whiten(sp.data_ptr(), n // 2)
        s.search_spectra([sp.data_ptr()], [n // 2], [rlo])
        staged = s.candidates()
        s.search([x], DT)
        assert np.array_equal(s.candidates(), staged) and len(staged) > 0
    orc = O.Oracle(50, 4, 2 * half)
    try:
        hi, lo = oracle_bounds(orc, w, rlo, 0, nsteps, cuts)
    finally:
        orc.close()
    g = keys(gpu, rlo, half, -50)
    assert len(g) > 0 and hi <= g <= lo
    best = gpu[np.argmax(gpu["power"])]
    assert abs(best["r"] - 20020.25) <= 1.0 and abs(best["z"] - 40) <= 4


def test_zmax300_request_through_the_server_matches_oracle():
    # the serving bank with the widest templates: zmax 300, 8 harmonics,
    # 8192-point segments; one request of 2^20 samples with a signal, served
    # by accel_server, equal to the context path, whose candidates equal the
    # oracle's on every step
    from gpu_accelsearch_gb300.search import AccelSearch, first_bin
    from gpu_accelsearch_gb300.serving import Server
    n = 1 << 20
    x = synth_series(n, seed=300300, signals=[(0.05, 123456.25, -120.0), (0.03, 401234.75, 250.0)])
    with Server(hbm_budget_bytes=4e9, fftlen=8192, numharm=8, chunk_segments=64) as srv:
        rid = srv.submit(x, DT, 300)
        assert srv.wait(rid, 300)
        served, _ = srv.result(rid)
    rlo = first_bin(n, DT)
    with AccelSearch(zmax=300, numharm=8, fftlen=8192) as s:
        s.search([x], DT)
        ctx = s.candidates()
        xd = torch.from_numpy(x).cuda()
        sp = torch.zeros((n // 2 + 1) * 2, dtype=torch.float32, device="cuda")
        s.rfft(xd.data_ptr(), n, sp.data_ptr())
        s.whiten(sp.data_ptr(), n // 2)
        s.search_spectra([sp.data_ptr()], [n // 2], [rlo])
        staged = s.candidates()
        w = host_c64(sp)[: n // 2]
        cuts = s.power_cuts().astype(np.float64)
        nsteps = s.step_count(n, DT)
        U = s.uselen
    for f in ("step", "r", "z", "numharm", "power", "sigma"):
        assert np.array_equal(served[f], ctx[f]), f
    assert np.array_equal(ctx, staged)
    orc = O.Oracle(300, 8, U)
    try:
        hi, lo = oracle_bounds(orc, w, rlo, 0, nsteps, cuts)
    finally:
        orc.close()
    g = keys(ctx, rlo, U // 2, -300)
    assert len(g) > 0 and hi <= g <= lo
    one = ctx[ctx["numharm"] == 1]
    for r0, z in ((123456.25, -120.0), (401234.75, 250.0)):
        near = one[np.abs(one["r"] - (r0 + z / 2)) < 20]
        assert len(near) > 0, (r0, z)
        b = near[np.argmax(near["power"])]
        assert abs(b["r"] - (r0 + z / 2)) <= 1.0 and abs(b["z"] - z) <= 4, (b, r0, z)
