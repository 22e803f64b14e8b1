"""The persistent plane-and-sum launch (accel_tuning.persistent: a launch
group's plane rows and harmonic-sum tiles from one work queue in one
kernel, k_step) against the separate kernels, through the C ABI: the same
float operations in the same order, so the candidate sets must be
bit-identical -- at ~3.5 sigma cuts (thousands of candidates), over launch
groups of 1 to 64 segments, FP32 and FP16 templates, graph and direct
launches, and a batch of uneven trials.  The separate tiled sum at tile
heights of 8, 16 and 32 rows, with tensor-map box copies or per-row bulk
copies, gives the same candidates too.  Its bounded waits are tested
without a GPU fault: with tuning.wait_test every tile's copy wait runs out,
the search fails with ACCEL_ERR_CUDA and the context recovers."""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
DT = 64e-6


def whitened(n, seed, sig):
    x = synth_series(n, seed=seed, signals=[sig])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
    return x, O.deredden(spec)


def search(s, d, nb, rlo, **tun):
    s.set_tuning(**tun)
    s.reset_stats()
    s.search_spectra([d.data_ptr()], [nb], [rlo])
    return s.candidates(), s.stats()["kinds"]["step"]["launches"]


@pytest.mark.parametrize("zmax,numharm", [(50, 4), (200, 8), (300, 8), (100, 16)])
def test_persistent_equals_separate_kernels(zmax, numharm):
    from gpu_accelsearch_gb300.search import AccelSearch
    n = 1 << 19
    _, w = whitened(n, 500 + zmax + numharm, (0.05, 40000.25, 30.0))
    d = torch.from_numpy(w.view(np.float32).copy()).cuda()
    with AccelSearch(zmax=zmax, numharm=numharm, fftlen=8192) as s:
        s.set_power_cuts(np.array([O.power_cut(3.5, 1 << k) for k in range(s.nstages)], np.float32))
        base, nstep = search(s, d, w.size, 16, chunk_segments=16, persistent=0)
        assert nstep == 0 and len(base) > 1000
        for chunk in (1, 7, 64):
            got, nstep = search(s, d, w.size, 16, chunk_segments=chunk, persistent=1)
            if numharm == 16:  # a 16-harmonic bank has segment lengths below 1024: separate kernels
                continue
            assert nstep > 0, chunk
            assert np.array_equal(got, base), chunk
        # and the separate tiled sum at its other tile heights, with its
        # rectangles brought in by tensor-map boxes (default) or row copies
        for rows in (8, 16, 32):
            for row_copies in (0, 1):
                got, _ = search(s, d, w.size, 16, chunk_segments=16, persistent=0, hsum_tile_rows=rows,
                                hsum_row_copies=row_copies)
                assert np.array_equal(got, base), (rows, row_copies)
        s.set_tuning(hsum_tile_rows=16, hsum_row_copies=0)


def test_persistent_fp16_graph_direct_and_batches():
    from gpu_accelsearch_gb300.search import AccelSearch
    n = 1 << 20
    x1, _ = whitened(n, 71, (0.05, 123456.25, -60.0))
    x2 = synth_series(3 << 18, seed=72, signals=[(0.08, 50000.5, 40.0)])
    for fp16 in (False, True):
        with AccelSearch(zmax=200, numharm=8, fftlen=8192, template_fp16=fp16) as s:
            s.set_tuning(chunk_segments=64, persistent=0)
            s.search([x1, x2], DT)
            base = s.candidates()
            for graph in (1, 0):
                s.set_tuning(persistent=1, graph=graph)
                s.reset_stats()
                s.search([x1, x2], DT)
                assert s.stats()["kinds"]["step"]["launches"] > 0
                assert np.array_equal(s.candidates(), base), (fp16, graph)
                xd = [torch.from_numpy(x).cuda() for x in (x1, x2)]
                s.search([t.data_ptr() for t in xd], DT, on_device=True, nsamples=[x1.size, x2.size])
                assert np.array_equal(s.candidates(), base), (fp16, graph, "device")


def test_persistent_wait_timeout_reported_and_context_recovers():
    from gpu_accelsearch_gb300.native import AccelError
    from gpu_accelsearch_gb300.search import AccelSearch
    n = 1 << 18
    x = synth_series(n, seed=9, signals=[(0.3, 5000.25, 20.0)])
    xd = torch.from_numpy(x.copy()).cuda()
    with AccelSearch(zmax=50, numharm=4, fftlen=8192) as s:
        s.set_tuning(chunk_segments=16, persistent=1, wait_test=0)
        s.search([x], DT)
        want = s.candidates()
        assert len(want) > 0 and s.stats()["kinds"]["step"]["launches"] > 0
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
