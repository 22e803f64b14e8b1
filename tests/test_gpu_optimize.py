"""Candidate refinement and properties (accel_optimize_candidates) against
the oracle's restatement (oracle.optimize / oracle.step_norms), through the
C ABI, at zmax 50 / 4 harmonics / L 2048:
  * without refinement the fundamental's power at a candidate's own cell is
    the search's power (the plane value) to 1e-4 of max(P, 1);
  * refined positions equal the oracle's to the finest grid step (1/64 bin,
    1/16 in z) and powers to 1e-4 relative;
  * refinement moves the injected signal towards its true (r, z);
  * f, fdot, period and pdot follow from r, z and the observation time.
"""
import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N, DT, RLO = 1 << 18, 64e-6, 16
R0, Z0 = 20000.25 + 0.3, 39.4   # off the search grid on purpose


@pytest.fixture(scope="module")
def run():
    from gpu_accelsearch_gb300.search import AccelSearch
    x = synth_series(N, seed=1018, signals=[(0.05, R0, Z0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)[: N // 2]
    w = O.deredden(spec)
    s = AccelSearch(zmax=50, numharm=4, fftlen=2048)
    d = torch.from_numpy(w.view(np.float32).copy()).cuda()
    s.search_spectra([d.data_ptr()], [w.size], [RLO])
    c = s.candidates()
    # the strongest candidates of every stage, plus some weak ones
    picks = []
    for nh in (1, 2, 4):
        cc = c[c["numharm"] == nh]
        picks += list(cc[np.argsort(-cc["power"])[:6]])
        picks += list(cc[:2])
    cands = np.array(picks, dtype=c.dtype)
    yield {"s": s, "w": w, "d": d, "c": cands}
    s.close()


def _opt(run, refine):
    s, w, d = run["s"], run["w"], run["d"]
    return s.optimize(run["c"], RLO, N * DT, spectra=[(d.data_ptr(), w.size)], refine=refine)


def test_unrefined_fundamental_equals_search_power(run):
    got = _opt(run, False)
    one = run["c"]["numharm"] == 1
    assert one.sum() >= 6
    p, want = got["power"][one].astype(np.float64), run["c"]["power"][one].astype(np.float64)
    assert np.all(np.abs(p - want) / np.maximum(want, 1.0) < 1e-4)
    assert np.array_equal(got["r"], run["c"]["r"]) and np.array_equal(got["z"], run["c"]["z"])


@pytest.mark.parametrize("refine", [False, True])
def test_matches_oracle(run, refine):
    got = _opt(run, refine)
    w, U = run["w"], run["s"].uselen
    for g, c in zip(got, run["c"]):
        H = int(c["numharm"])
        norms = O.step_norms(w, 50, 4, U, RLO, int(c["step"]), H)
        r, z, p, hp = O.optimize(w, float(c["r"]), float(c["z"]), H, norms, refine=refine)
        assert abs(g["r"] - r) <= 1 / 64 + 1e-12 and abs(g["z"] - z) <= 1 / 16 + 1e-12, (c, g, r, z)
        if g["r"] == r and g["z"] == z:
            assert abs(g["power"] - p) / max(p, 1.0) < 1e-4
            assert np.all(np.abs(g["harm_power"][:H] - hp) / np.maximum(hp, 1.0) < 1e-4)
        assert g["r_grid"] == c["r"] and g["z_grid"] == c["z"]


def test_refinement_approaches_the_signal(run):
    got = _opt(run, True)
    c = run["c"]
    one = np.nonzero(c["numharm"] == 1)[0]
    k = one[np.argmax(c["power"][one])]
    rs = R0 + Z0 / 2  # the signal's mean frequency
    assert abs(c["r"][k] - rs) <= 0.5
    assert abs(got["r"][k] - rs) < 0.1 and abs(got["z"][k] - Z0) < 1.0
    assert got["power"][k] >= c["power"][k]
    T = N * DT
    f, fd = got["r"][k] / T, got["z"][k] / T ** 2
    assert np.isclose(got["f"][k], f) and np.isclose(got["fdot"][k], fd)
    assert np.isclose(got["period"][k], 1 / f) and np.isclose(got["pdot"][k], -fd / f ** 2)
