"""The FP32 CPU restatement used as the CPU baseline (oracle/cpu_fp32.py)
against the FP64 oracle: stage sums of whole steps of the small
configuration (zmax 50, 4 harmonics, L 2048) within |P - P64| / max(P64, 1)
< 1e-4, and the same steps through the spawn process pool."""
import numpy as np

from gpu_accelsearch_gb300.synth import synth_series
from oracle import cpu_fp32 as F
from oracle import oracle as O


def test_fp32_port_stage_sums_match_oracle():
    n = 1 << 18
    x = synth_series(n, seed=1018, signals=[(0.05, 20000.25, 40.0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
    w = O.deredden(spec)
    s = F.Fp32Search(50, 4, 1914)
    orc = O.Oracle(50, 4, 1914)
    try:
        for k in (0, 20, 135):
            got = s.step(w, 16 + k * 957)
            _, planes, _ = orc.run_steps(w, 16, k, 1, want_planes=True)
            err = (np.abs(got - planes[0]) / np.maximum(planes[0], 1.0)).max()
            assert err < 1e-4, (k, err)
    finally:
        orc.close()


def test_fp32_port_process_pool():
    n = 1 << 18
    x = synth_series(n, seed=1018, signals=[(0.05, 20000.25, 40.0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: n // 2]
    w = O.deredden(spec)
    cuts = np.array([O.power_cut(6.0, 1 << k) for k in range(3)])
    el, nc, procs = F.timed_search(50, 4, 1914, w, [16 + 957 * k for k in range(8)], cuts, processes=2)
    assert el > 0 and procs == 2
    s = F.Fp32Search(50, 4, 1914)
    want = sum(int(np.count_nonzero(s.step(w, 16 + 957 * k)[j] > cuts[j])) for k in range(8) for j in range(3))
    assert nc == want
