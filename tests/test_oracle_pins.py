"""The CPU oracle against values produced by the reference's own host code.

tests/golden/reference_pins.json was written by tests/golden/make_golden.py
from the reference's sources (bpd_math.c, bpd_noise.c, bpd_fresnl.c,
bpd_subharmonics.cu, bpd_search.cu) compiled by oracle/ref/Makefile.  All
comparisons here are bit-exact: the oracle restates those host routines
operation for operation.
"""
import hashlib

import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_red_spectrum, synth_series
from oracle import oracle as O


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_rsqrt_magic(pins):
    xs = np.linspace(0.0, 40.0, 4001, dtype=np.float32)
    assert sha(xs) == pins["rsqrt"]["x_sha"]
    ys = np.array([O.rsqrt_magic(float(x)) for x in xs], np.float32)
    assert sha(ys) == pins["rsqrt"]["y_sha"]


def test_fresnel(pins):
    for x, (s, c) in zip(pins["fresnl"]["x"], pins["fresnl"]["sc"]):
        assert O.fresnl(x) == (s, c), x


def test_halfwidth_and_required(pins):
    for z, m in pins["z_halfwidth"].items():
        assert O.z_halfwidth(float(z)) == m, z
    for kind, h, H, v, want in pins["calc_required"]:
        f = h / H
        got = O.calc_required_z(f, v) if kind == "z" else O.calc_required_r(f, v)
        assert got == want, (kind, h, H, v)


def test_responses(pins):
    for key, rec in pins["responses"].items():
        if key.startswith("r_response"):
            got = O.r_response(64, roffset=0.25).view(np.float32)
        else:
            got = O.z_response(float(key), rec["numkern"]).view(np.float32)
        assert sha(got) == rec["sha"], key


def test_median(pins):
    rng = np.random.default_rng(7)
    for rec in pins["median_seeded"]:
        n = rec["n"]
        a = rng.exponential(1.0, n).astype(np.float32)
        if n > 10:
            a[: n // 5] = a[n // 3]
        assert sha(a) == rec["a_sha"]
        assert O.lower_median(a) == np.float32(rec["m"])


def test_deredden(pins):
    rec = pins["deredden"]
    spec = synth_red_spectrum(rec["numbins"], seed=rec["seed"])
    assert sha(spec) == rec["in_sha"], "synthetic generator changed"
    assert sha(O.deredden(spec)) == rec["out_sha"]


def test_deredden_short_spectra_and_nan_tail(pins):
    # the reference's whitening of short spectra; at 5220 bins the last
    # slope drives the extrapolated tail level below zero and the reference
    # itself gives NaN there (the oracle and the GPU follow it)
    for rec in pins["deredden_tails"]:
        n = rec["numbins"]
        spec = synth_red_spectrum(n + 1, seed=rec["seed"])[:n]
        assert sha(spec) == rec["in_sha"], "synthetic generator changed"
        w = O.deredden(spec)
        f = w.view(np.float32)
        assert np.nonzero(np.isnan(f))[0].tolist() == rec["nan_floats"]
        assert sha(w) == rec["out_sha"], n
    assert any(rec["nan_floats"] for rec in pins["deredden_tails"])


@pytest.mark.parametrize("bank_index", range(7))
def test_bank(pins, bank_index):
    rec = pins["banks"][bank_index]
    geom = O.bank_geometry(rec["zmax"], rec["numharm"], rec["uselen"])
    assert len(geom) == len(rec["harmonics"])
    for h, hr in enumerate(rec["harmonics"]):
        info = hr["info"]  # harmnum, maxharm, zmax, numzs, fftlen, hw0
        assert list(geom[h, :6]) == info
        if rec["uselen"] > 16000:
            continue  # the 32K bank is pinned on geometry only (size)
        numzs, L, zm = info[3], info[4], info[2]
        bank = np.concatenate([O.wrapped_template(L, -zm + 2 * j) for j in range(numzs)])
        assert sha(bank.view(np.float32)) == hr["templates_sha"], (bank_index, h)


@pytest.mark.parametrize("which", [0, 1])
def test_step_geometry_and_segments(pins, which):
    rec = pins["steps"][which]
    zmax, numharm, U = rec["zmax"], rec["numharm"], rec["uselen"]
    n = 1 << rec["nlog2"]
    x = synth_series(n, seed=rec["series_seed"], signals=[(0.05, 20000.25, 40.0)])
    assert sha(x) == rec["series_sha"], "synthetic generator changed"
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)
    w = O.deredden(spec[: n // 2])
    assert sha(w) == rec["whitened_sha"]
    assert O.step_count(n // 2, rec["rlo"], U) == rec["nsteps"]
    geom = O.bank_geometry(zmax, numharm, U)
    for st in rec["steps"][:: 7 if which == 0 else 1]:
        startr = st["startr"]
        lastr = startr + U // 2 - 0.5
        segs = []
        for h, g in enumerate(geom):
            rlo, rhi, zlo, numrs = O.step_ffdot(int(g[0]), int(g[1]), zmax, U, startr, lastr)
            want = st["ffdot"][6 * h: 6 * h + 6]  # rlo, numrs, numzs, fftlen, zlo, binoffset
            assert [rlo, numrs, int(g[3]), int(g[4]), zlo, int(g[5])] == want
            assert rhi == st["rhi"][h]
            segs.append(O.segment_data(w, rlo, rhi, int(g[5]), int(g[4])))
        assert sha(np.concatenate(segs).view(np.float32)) == st["data_sha"], st["step"]


def test_exact_rsqrt_mode_switch():
    # the oracle's exact mode is IEEE 1/sqrtf; the default stays the
    # reference's magic-constant rsqrt, and the switch is reversible
    xs = np.linspace(0.01, 40.0, 997, dtype=np.float32)
    magic = np.array([O.rsqrt_magic(float(x)) for x in xs], np.float32)
    assert np.array_equal(np.array([O.rsqrt_norm(float(x)) for x in xs], np.float32), magic)
    O.set_exact_rsqrt(True)
    try:
        got = np.array([O.rsqrt_norm(float(x)) for x in xs], np.float32)
        spec = synth_red_spectrum(1 << 14, seed=3)
        w_exact = O.deredden(spec)
    finally:
        O.set_exact_rsqrt(False)
    assert np.array_equal(got, np.float32(1.0) / np.sqrt(xs))
    rel = np.abs(magic.astype(np.float64) / got - 1)
    assert 1e-4 < rel.max() < 2e-3
    w_magic = O.deredden(spec)
    assert not np.array_equal(w_exact, w_magic)
    assert np.abs(np.abs(w_exact) / np.abs(w_magic) - 1)[1:].max() < 2e-3


def test_oracle_planes_equal_reference_kernels():
    # the oracle's FP64 restatement of convolveSignal / inverse FFT /
    # generatePowers / addPowers against the reference's own kernel source
    # run on the host (tests/golden/reference_planes.npz): fundamental powers
    # and every harmonic stage sum of one step, over the stored columns
    import golden_planes as GP
    g = GP.load()
    for case, step, zmax, numharm, uselen, numbins, startr, (c0, c1), ref in GP.cases(g):
        w = GP.spectrum(g, case, step, numbins)
        orc = O.Oracle(zmax, numharm, uselen)
        try:
            rlo = int(g[case + "_meta"][5])
            k = (startr - rlo) // (uselen // 2)
            _, planes, _ = orc.run_steps(w, rlo, k, 1, want_planes=True)
        finally:
            orc.close()
        got = planes[0][:, :, c0:c1]
        assert got.shape == ref.shape, (case, step)
        err = (np.abs(got - ref) / np.maximum(ref, 1.0)).max()
        assert err < 2e-6, (case, step, err)
