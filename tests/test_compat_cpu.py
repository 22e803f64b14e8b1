"""Host-side drop-in functions (include/bpd_compat.h) against values the
reference's own code produced (tests/golden/reference_pins.json): the step
geometry of generate_harmonics_ffdot and the spread segments of
generate_harmonic_ffdot_data, bit for bit.  No GPU needed."""
import ctypes as C
import hashlib

import numpy as np
import pytest

import __graft_entry__
from gpu_accelsearch_gb300 import compat as CP
from gpu_accelsearch_gb300.synth import synth_series
from oracle import oracle as O


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def L():
    __graft_entry__.build_library()
    return CP.lib()


def make_shi(zmax, numharm, U):
    geom = O.bank_geometry(zmax, numharm, U)
    nh = len(geom)
    shi = (CP.SubharmonicInfo * nh)()
    keep = []
    for h, g in enumerate(geom):
        hw = (C.c_ushort * int(g[3]))(*[O.z_halfwidth(-int(g[2]) + 2 * j) for j in range(int(g[3]))])
        keep.append(hw)
        shi[h].maxHarmonic, shi[h].currentHarmonic, shi[h].zmax = int(g[1]), int(g[0]), int(g[2])
        shi[h].totalKernelsTemplates, shi[h].kernelFFTLength = int(g[3]), int(g[4])
        shi[h].kernelHalfWidth = C.cast(hw, C.POINTER(C.c_ushort))
    return shi, keep, geom


@pytest.mark.parametrize("which", [0, 1])
def test_segment_preparation_matches_reference(L, pins, which):
    rec = pins["steps"][which]
    zmax, numharm, U = rec["zmax"], rec["numharm"], rec["uselen"]
    L.accel_compat_set_uselen(U)
    stages = int(np.log2(numharm)) + 1
    shi, keep, geom = make_shi(zmax, numharm, U)
    nh = len(geom)
    n = 1 << rec["nlog2"]
    x = synth_series(n, seed=rec["series_seed"], signals=[(0.05, 20000.25, 40.0)])
    spec = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)
    w = O.deredden(spec[: n // 2])
    assert sha(w) == rec["whitened_sha"]
    starts = (C.c_long * nh)()
    tot = 0
    for h in range(nh):
        starts[h] = tot
        tot += int(geom[h, 4])
    out = np.zeros(tot, np.complex64)
    fi = (CP.FfdotInfo * nh)()
    bo = (C.c_ushort * nh)()
    for st in rec["steps"][:: 9 if which == 0 else 1]:
        startr = st["startr"]
        L.generate_harmonics_ffdot(nh, stages, shi, startr, startr + U // 2 - 0.5, -zmax, fi, bo)
        got = []
        for h in range(nh):
            got += [fi[h].rlo, fi[h].numrs, fi[h].numzs, fi[h].fftlen, fi[h].zlo, bo[h]]
            assert fi[h].rhi == st["rhi"][h]
        assert got == st["ffdot"]
        L.generate_harmonic_ffdot_data(nh, tot, fi, bo, starts, w.ctypes.data, w.size, 0,
                                       out.ctypes.data)
        assert L.accel_compat_status() == 0
        assert sha(out.view(np.float32)) == st["data_sha"], st["step"]
    L.accel_compat_set_uselen(32000)


def test_required_and_indices(L, pins):
    for kind, h, H, v, want in pins["calc_required"]:
        f = h / H
        got = L.calc_required_z(f, v) if kind == "z" else L.calc_required_r(f, v)
        assert got == want
    assert L.getTotalHarmonics(4) == 8
    assert L.index_from_r(20000.5, 20000.0) == 1 and L.index_from_z(-48.0, -50.0) == 1


def test_read_data_padding_and_limits(L, tmp_path):
    # readData (bpd_data.c:9-75): samples behind 2000 zero samples, 2000 zeros
    # after them, at most 2^26 samples; errors come back as a status
    x = np.random.default_rng(5).standard_normal(12345).astype(np.float32)
    f = tmp_path / "series.dat"
    x.tofile(f)
    p = C.POINTER(C.c_float)()
    n = L.readData(str(f).encode(), C.byref(p))
    assert L.accel_compat_status() == 0 and n == x.size
    base = C.cast(C.addressof(p.contents) - 2000 * 4, C.POINTER(C.c_float))
    buf = np.ctypeslib.as_array(base, shape=(n + 4000,)).copy()
    L.freeData(p)
    assert np.array_equal(buf[2000:2000 + n], x)
    assert not buf[:2000].any() and not buf[2000 + n:].any()
    empty = tmp_path / "empty.dat"
    empty.write_bytes(b"")
    assert L.readData(str(empty).encode(), C.byref(p)) == 0 and L.accel_compat_status() < 0
    big = tmp_path / "big.dat"
    with open(big, "wb") as fh:
        fh.truncate(((1 << 26) + 1) * 4)  # sparse: one sample over the limit
    assert L.readData(str(big).encode(), C.byref(p)) == 0 and L.accel_compat_status() < 0
    assert L.readData(str(tmp_path / "missing.dat").encode(), C.byref(p)) == 0
    assert L.accel_compat_status() < 0
