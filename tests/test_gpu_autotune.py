"""The autotuner (accel_autotune) through the C ABI: it returns a
configuration that builds, its choice lies in the candidate set it was
given, and a search with the tuned configuration gives exactly the
candidates of the same configuration set by hand (and of the default
launch shape at that segment length), equal to the FP64 oracle's outside
the +-1e-4 band around each cut."""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series
from oracle import oracle as O
from parity_keys import keys, oracle_bounds

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DT = 64e-6


def test_autotuned_configuration_searches_like_the_hand_set_one():
    from gpu_accelsearch_gb300.search import AccelSearch, autotune, first_bin
    lens = (2048, 4096)
    kw, tun, rate = autotune(zmax=50, numharm=4, fftlens=lens, steps=48)
    assert kw["fftlen"] in lens and rate > 0
    assert tun["chunk_segments"] in (16, 32, 64, 128, 256, 512)
    assert tun["plane_split"] in (0, 1) and tun["fused_sum"] in (0, 1)
    assert tun["hsum_tile_rows"] in (8, 16, 32)
    n = 1 << 18
    x = synth_series(n, seed=77, signals=[(0.05, 30000.25, -24.0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
    w = O.deredden(spec)
    rlo = first_bin(n, DT)
    d = torch.from_numpy(w.view(np.float32).copy()).cuda()
    with AccelSearch(**kw) as s:
        s.set_tuning(**tun)
        assert {k: s.tuning()[k] for k in tun} == tun
        s.search_spectra([d.data_ptr()], [w.size], [rlo])
        tuned = s.candidates()
        cuts = s.power_cuts().astype(np.float64)
        U = s.uselen
        nsteps = s.step_count(n, DT)
    with AccelSearch(zmax=50, numharm=4, fftlen=kw["fftlen"], chunk_segments=tun["chunk_segments"]) as s:
        s.set_tuning(chunk_segments=tun["chunk_segments"], plane_split=tun["plane_split"],
                     fused_sum=tun["fused_sum"], hsum_tile_rows=tun["hsum_tile_rows"])
        s.search_spectra([d.data_ptr()], [w.size], [rlo])
        by_hand = s.candidates()
    with AccelSearch(zmax=50, numharm=4, fftlen=kw["fftlen"]) as s:
        s.search_spectra([d.data_ptr()], [w.size], [rlo])
        default = s.candidates()
    assert len(tuned) > 0
    assert np.array_equal(tuned, by_hand) and np.array_equal(tuned, default)
    orc = O.Oracle(50, 4, U)
    try:
        hi, lo = oracle_bounds(orc, w, rlo, 0, nsteps, cuts)
    finally:
        orc.close()
    assert hi <= keys(tuned, rlo, U // 2, -50) <= lo
