"""accel_whiten_noalloc -- whitening for callers that cannot allocate device
memory (real-time pipelines that size everything at start-up, plugins inside
another application's memory pool) -- checked through the C ABI against the
context path accel_whiten on two calls in a row.  Whitening is bit-exact, so
the tolerance is zero.  This file sorts last so that a run stopping at the
first failure has run every other test already."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _noalloc():
    from gpu_accelsearch_gb300 import native as N
    L = N.lib()
    f = L.accel_whiten_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p]
    return L, f


def _context_whiten(spec, numbins, init, maxb):
    from gpu_accelsearch_gb300.search import AccelSearch
    d = torch.from_numpy(spec.view(np.float32).copy()).cuda()
    with AccelSearch(zmax=50, numharm=4, fftlen=2048, whiten_initbuf=init, whiten_maxbuf=maxb) as s:
        s.whiten(d.data_ptr(), numbins)
        s.synchronize()
    return d.cpu().numpy()


def test_noalloc_whitening_matches_context_path():
    from gpu_accelsearch_gb300.synth import synth_red_spectrum
    L, whiten = _noalloc()
    # the warp-per-block kernels (blocks of at most 1024 bins) and the
    # CTA-per-block kernels with opt-in shared memory (blocks of 4096 bins)
    cases = [(1 << 17, 6, 200, 31), (40001, 1000, 1000, 32), (1 << 20, 600, 4096, 33)]
    for numbins, init, maxb, seed in cases:
        spec = synth_red_spectrum(numbins + 1, seed=seed)
        want = _context_whiten(spec, numbins, init, maxb)
        for _ in range(2):  # two calls in a row share the static scratch
            d = torch.from_numpy(spec.view(np.float32).copy()).cuda()
            torch.cuda.synchronize()
            rc = whiten(d.data_ptr(), numbins, init, maxb, None)
            assert rc == 0, L.accel_last_error().decode()
            torch.cuda.synchronize()
            got = d.cpu().numpy()
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_noalloc_rejects_oversize():
    L, whiten = _noalloc()
    d = torch.zeros(2, dtype=torch.float32, device="cuda")
    rc = whiten(d.data_ptr(), 1 << 30, 6, 200, None)
    assert rc == -1
    assert "static scratch" in L.accel_last_error().decode()


def test_noalloc_refused_inside_stream_capture():
    # the block table is copied from host arrays that the next call
    # rewrites, so a captured call is refused and nothing is enqueued
    L, whiten = _noalloc()
    d = torch.zeros(2 * 4096, dtype=torch.float32, device="cuda")
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            d.add_(1.0)
            rc = whiten(d.data_ptr(), 4000, 6, 200, torch.cuda.current_stream().cuda_stream)
    assert rc == -5
    assert "capture" in L.accel_last_error().decode()
    g.replay()
    torch.cuda.synchronize()
    assert float(d[0]) == 1.0
