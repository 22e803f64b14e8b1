"""Edge cases of the search through the C ABI: an empty batch, a trial too
short for one overlap-save step beside normal ones, odd sample counts, a
candidate buffer that overflows, a bank of one template (zmax 0) and a
single-harmonic search -- the last two against the FP64 oracle."""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DT = 64e-6
TOL_P = 1e-4


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.float32).copy()).cuda()


def _keys(a, rlo, half, zlo0):
    if "ridx" in a.dtype.names:
        return {(int(c["step"]), int(c["ridx"]), int(c["zidx"]), int(c["numharm"])) for c in a}
    return {(int(c["step"]), int(round(2 * (c["r"] - (rlo + c["step"] * half)))),
             int(round((c["z"] - zlo0) / 2)), int(c["numharm"])) for c in a}


@pytest.fixture(scope="module")
def S():
    from gpu_accelsearch_gb300.search import AccelSearch
    s = AccelSearch(zmax=50, numharm=4, fftlen=2048)
    yield s
    s.close()


def test_empty_batch(S):
    assert S.search([], DT) == 0
    assert len(S.candidates()) == 0


def test_short_trial_beside_normal_ones(S):
    # a 2^10-sample trial has no overlap-save step at this segment length;
    # it neither fails nor changes the other trials' candidates
    x = synth_series(1 << 18, seed=5, signals=[(0.05, 30000.25, 20.0)])
    tiny = synth_series(1 << 10, seed=6)
    assert S.step_count(1 << 10, DT) == 0
    S.search([x], DT)
    alone = S.candidates()
    S.search([tiny, x, tiny], DT)
    mix = S.candidates()
    assert set(mix["trial"]) <= {1}
    mine = mix.copy()
    mine["trial"] = 0
    key = ["step", "numharm", "z", "r"]
    assert len(alone) > 0
    assert np.array_equal(np.sort(alone, order=key), np.sort(mine, order=key))


def test_odd_sample_count_rejected(S):
    from gpu_accelsearch_gb300 import native as N
    with pytest.raises(N.AccelError) as e:
        S.search([synth_series((1 << 16) + 1, seed=1)], DT)
    assert e.value.code == -1


def test_candidate_overflow_reports_capacity():
    from gpu_accelsearch_gb300 import native as N
    from gpu_accelsearch_gb300.search import AccelSearch
    x = synth_series(1 << 18, seed=7)
    with AccelSearch(zmax=50, numharm=4, fftlen=2048, cand_capacity=1000) as s:
        s.set_power_cuts(np.array([3.0, 5.0, 8.0], np.float32))  # far below noise
        with pytest.raises(N.AccelError) as e:
            s.search([x], DT)
        assert e.value.code == -4
        assert len(s.candidates()) == 1000  # the buffer's worth is still returned


@pytest.mark.parametrize("zmax,numharm", [(0, 4), (50, 1)])
def test_small_banks_match_oracle(zmax, numharm):
    from gpu_accelsearch_gb300.search import AccelSearch
    n = 1 << 18
    x = synth_series(n, seed=11, signals=[(0.06, 25000.25, float(zmax // 2))])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
    w = O.deredden(spec)
    with AccelSearch(zmax=zmax, numharm=numharm, fftlen=2048) as s:
        cuts = np.array([O.power_cut(3.0, 1 << k) for k in range(s.nstages)])
        s.set_power_cuts(cuts.astype(np.float32))
        d = dev(w)
        s.search_spectra([d.data_ptr()], [w.size], [16])
        gpu = s.candidates()
        o = O.Oracle(zmax, numharm, s.uselen)
        try:
            steps = 12
            gpu = gpu[gpu["step"] < steps]
            c32 = cuts.astype(np.float32).astype(np.float64)
            lo, _, _ = o.run_steps(w, 16, 0, steps, powcut=c32 * (1 - TOL_P), cap=1 << 22)
            hi, _, _ = o.run_steps(w, 16, 0, steps, powcut=c32 * (1 + TOL_P), cap=1 << 22)
        finally:
            o.close()
        g = _keys(gpu, 16, s.uselen // 2, -zmax)
        assert len(g) > 20
        assert _keys(hi, 0, 0, 0) <= g <= _keys(lo, 0, 0, 0)


def test_tile_wait_timeout_reported_and_context_recovers():
    # failure detection without a GPU fault: with tuning.wait_test every tile
    # of the harmonic sum waits for 16 bytes that never arrive, so its bounded
    # wait runs out, it sets the error word and returns; the search (host-fed,
    # and from device series through the CUDA graph) fails with
    # ACCEL_ERR_CUDA, and the same context then searches normally
    from gpu_accelsearch_gb300.native import AccelError
    from gpu_accelsearch_gb300.search import AccelSearch
    n = 1 << 16
    x = synth_series(n, seed=9, signals=[(0.3, 5000.25, 20.0)])
    xd = torch.from_numpy(x.copy()).cuda()
    with AccelSearch(zmax=50, numharm=4, fftlen=2048) as s:
        s.set_tuning(hsum_pipelined=0, hsum_rowwise=0, wait_test=0)
        s.search([x], DT)
        want = s.candidates()
        assert len(want) > 0
        s.set_tuning(wait_test=1)
        for kw in ({}, {"on_device": True, "nsamples": [n]}):
            src = [xd.data_ptr()] if kw else [x]
            with pytest.raises(AccelError) as e:
                s.search(src, DT, **kw)
            assert e.value.code == -2 and "timed out" in str(e.value)
        s.set_tuning(wait_test=0)
        s.search([x], DT)
        assert np.array_equal(s.candidates(), want)
        s.search([xd.data_ptr()], DT, on_device=True, nsamples=[n])
        assert np.array_equal(s.candidates(), want)
