"""CUDA-graph launch of device-resident searches (accel_tuning.graph).

A search recorded into a CUDA graph runs the same kernels with the same
arguments as the direct launches, so its candidates must be bit-identical:
on repeated searches of the same shape (the kept executable graph updated in
place, no new instantiation), after the shape changes (another trial set or
launch-group size: instantiated anew), with the harmonic sum overlapped on
the second stream or serial, and with per-kernel profiling on (the timing
events become event-record nodes of the graph).  Searches from host series
launch directly even with the option set.
"""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CUTS = np.array([6.6, 9.2, 13.1], np.float32)  # ~3 sigma: many candidates


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.float32).copy()).cuda()


@pytest.fixture(scope="module")
def trials():
    out = []
    for i, n in enumerate([1 << 18, 3 << 16, 1 << 17]):
        x = synth_series(n, seed=4100 + i, signals=[(0.05, 9000.25 + 1000 * i, 30.0)])
        spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
        out.append({"n": n, "x": x, "w": O.deredden(spec), "rlo": 16})
    return out


def _search(s, devs, trials, k):
    s.search_spectra([d.data_ptr() for d in devs[:k]], [t["w"].size for t in trials[:k]],
                     [t["rlo"] for t in trials[:k]])
    return s.candidates()


@pytest.mark.parametrize("serial", [0, 1])
def test_graph_matches_direct(trials, serial):
    from gpu_accelsearch_gb300.search import AccelSearch
    devs = [dev(t["w"]) for t in trials]
    with AccelSearch(zmax=50, numharm=4, fftlen=2048) as s:
        s.set_power_cuts(CUTS)
        s.set_tuning(chunk_segments=48, serial_sum=serial, graph=0)
        want3 = _search(s, devs, trials, 3)
        want2 = _search(s, devs, trials, 2)
        assert len(want3) > 10000
        s.set_tuning(graph=1)
        assert s.tuning()["graph"] == 1
        s.reset_stats()
        for _ in range(2):  # the second search updates the kept graph
            assert np.array_equal(_search(s, devs, trials, 3), want3)
        st = s.stats()
        assert st["graph_launches"] == 2 and st["graph_builds"] == 1, st
        # another shape (fewer segments): instantiated anew, then reused
        assert np.array_equal(_search(s, devs, trials, 2), want2)
        assert np.array_equal(_search(s, devs, trials, 2), want2)
        st = s.stats()
        assert st["graph_launches"] == 4 and st["graph_builds"] == 2, st
        # another launch-group size, with the timing events inside the graph
        s.set_tuning(chunk_segments=31)
        s.profile(True)
        try:
            got = _search(s, devs, trials, 3)
        finally:
            s.profile(False)
        assert np.array_equal(got, want3)
        st = s.stats()
        assert st["graph_launches"] == 5
        assert st["kinds"]["plane"]["ms"] > 0 and st["kinds"]["hsum"]["ms"] > 0, st


def test_graph_series_on_device_and_host(trials):
    # series on the device: transformed and whitened first, then the graph;
    # series in host memory: copies interleaved with the groups, direct launches
    from gpu_accelsearch_gb300.search import AccelSearch
    t = trials[0]
    xd = torch.from_numpy(t["x"].copy()).cuda()
    with AccelSearch(zmax=50, numharm=4, fftlen=2048) as s:
        s.set_tuning(chunk_segments=48, graph=0)
        s.search([t["x"]], 64e-6)
        want = s.candidates()
        assert len(want) > 0
        s.set_tuning(graph=1)
        s.reset_stats()
        s.search([xd.data_ptr()], 64e-6, on_device=True, nsamples=[t["n"]])
        assert np.array_equal(s.candidates(), want)
        assert s.stats()["graph_launches"] == 1
        s.search([t["x"]], 64e-6)
        assert np.array_equal(s.candidates(), want)
        assert s.stats()["graph_launches"] == 1


def test_search_on_caller_stream(trials):
    # accel_set_stream: the search runs on the caller's stream, ordered after
    # the caller's still-pending kernels that produce its input (a spin of
    # about 0.1 s delays them), as a graph and as direct launches
    import ctypes as C

    from gpu_accelsearch_gb300 import native as N
    from gpu_accelsearch_gb300.search import AccelSearch
    t = trials[0]
    src = dev(t["w"])
    with AccelSearch(zmax=50, numharm=4, fftlen=2048) as s:
        s.set_power_cuts(CUTS)
        s.set_tuning(chunk_segments=48, graph=0)
        want = _search(s, [src], [t], 1)
        side = torch.cuda.Stream()
        torch.cuda.synchronize()
        for graph in (1, 0):
            s.set_tuning(graph=graph)
            with torch.cuda.stream(side):
                d = torch.zeros_like(src)
                if hasattr(torch.cuda, "_sleep"):
                    torch.cuda._sleep(200_000_000)
                d.copy_(src)
                N.check(N.lib().accel_set_stream(s._h, C.c_void_p(side.cuda_stream)))
                try:
                    got = _search(s, [d], [t], 1)
                finally:
                    N.check(N.lib().accel_set_stream(s._h, None))
            torch.cuda.synchronize()
            assert np.array_equal(got, want), graph
