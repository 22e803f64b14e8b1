"""SIGPROC filterbank reader (host only): files written here in the SIGPROC
layout (counted keyword strings, int32/float64/string values, time-major
samples) are read back channel-major with their header; unsupported or
broken files are refused with a status."""
import struct

import numpy as np
import pytest

import __graft_entry__
from gpu_accelsearch_gb300.dedisperse import read_filterbank
from gpu_accelsearch_gb300.native import AccelError


@pytest.fixture(scope="module", autouse=True)
def lib():
    __graft_entry__.build_library()


def _s(x: str) -> bytes:
    b = x.encode()
    return struct.pack("<i", len(b)) + b


def write_fil(path, data_tm, nbits, extra=b"", nchans=None, fch1=1510.0, foff=-0.5, tsamp=64e-6,
              nifs=1, start=b"HEADER_START"):
    nchans = data_tm.shape[1] if nchans is None else nchans
    h = struct.pack("<i", len(start)) + start
    h += _s("source_name") + _s("PSR_FAKE")
    h += _s("telescope_id") + struct.pack("<i", 6)
    h += _s("machine_id") + struct.pack("<i", 10)
    h += _s("data_type") + struct.pack("<i", 1)
    h += _s("fch1") + struct.pack("<d", fch1)
    h += _s("foff") + struct.pack("<d", foff)
    h += _s("nchans") + struct.pack("<i", nchans)
    h += _s("nbits") + struct.pack("<i", nbits)
    h += _s("tstart") + struct.pack("<d", 60000.25)
    h += _s("tsamp") + struct.pack("<d", tsamp)
    h += _s("nifs") + struct.pack("<i", nifs)
    h += extra + _s("HEADER_END")
    dt = {8: np.uint8, 16: np.uint16, 32: np.float32}[nbits]
    with open(path, "wb") as f:
        f.write(h)
        f.write(np.ascontiguousarray(data_tm, dtype=dt).tobytes())
    return len(h)


@pytest.mark.parametrize("nbits", [8, 16, 32])
def test_roundtrip(tmp_path, nbits):
    rng = np.random.default_rng(nbits)
    nt, nc = 10007, 48  # more samples than one read block, a ragged last block
    if nbits == 32:
        tm = rng.standard_normal((nt, nc)).astype(np.float32)
    else:
        tm = rng.integers(0, 1 << nbits, (nt, nc)).astype(np.float64)
    p = tmp_path / f"x{nbits}.fil"
    hb = write_fil(p, tm, nbits, extra=_s("src_raj") + struct.pack("<d", 123456.7))
    hdr, data = read_filterbank(p)
    assert data.shape == (nc, nt) and data.dtype == np.float32
    assert np.array_equal(data, tm.T.astype(np.float32))
    assert (hdr["nchans"], hdr["nbits"], hdr["nsamples"], hdr["header_bytes"]) == (nc, nbits, nt, hb)
    assert (hdr["fch1"], hdr["foff"], hdr["tsamp"], hdr["tstart"]) == (1510.0, -0.5, 64e-6, 60000.25)
    assert hdr["source_name"] == "PSR_FAKE"


def test_signed_8bit(tmp_path):
    # the one-byte "signed" keyword marks two's-complement 8-bit samples
    rng = np.random.default_rng(3)
    nt, nc = 5000, 16
    vals = rng.integers(-128, 128, (nt, nc)).astype(np.int8)
    p = tmp_path / "s8.fil"
    write_fil(p, vals.view(np.uint8), 8, extra=_s("signed") + b"\x01")
    hdr, data = read_filterbank(p)
    assert hdr["is_signed"] == 1
    assert np.array_equal(data, vals.T.astype(np.float32))
    # "signed" = 0 keeps unsigned samples
    write_fil(p, vals.view(np.uint8), 8, extra=_s("signed") + b"\x00")
    hdr, data = read_filterbank(p)
    assert hdr["is_signed"] == 0
    assert np.array_equal(data, vals.view(np.uint8).T.astype(np.float32))


def test_nsamples_keyword_limits_and_trailing_bytes_ignored(tmp_path):
    tm = np.arange(40 * 4, dtype=np.float32).reshape(40, 4)
    p = tmp_path / "n.fil"
    write_fil(p, tm, 32, extra=_s("nsamples") + struct.pack("<i", 25))
    hdr, data = read_filterbank(p)
    assert hdr["nsamples"] == 25 and np.array_equal(data, tm[:25].T)
    with open(p, "ab") as f:  # a partial time sample at the end
        f.write(b"\x01\x02")
    hdr, data = read_filterbank(p)
    assert hdr["nsamples"] == 25


@pytest.mark.parametrize("case", ["no_header", "unknown_keyword", "four_bit", "two_ifs", "truncated"])
def test_refused(tmp_path, case):
    tm = np.zeros((10, 4), np.float32)
    p = tmp_path / f"{case}.fil"
    if case == "no_header":
        write_fil(p, tm, 32, start=b"HEADER_BEGIN")
    elif case == "unknown_keyword":
        write_fil(p, tm, 32, extra=_s("mystery") + struct.pack("<i", 1))
    elif case == "four_bit":
        write_fil(p, np.zeros((10, 4), np.uint8), 8)
        raw = bytearray(p.read_bytes())
        i = raw.index(b"nbits") + 5
        raw[i:i + 4] = struct.pack("<i", 4)
        p.write_bytes(bytes(raw))
    elif case == "two_ifs":
        write_fil(p, tm, 32, nifs=2)
    else:
        n = write_fil(p, tm, 32)
        p.write_bytes(p.read_bytes()[: n - 6])
    with pytest.raises(AccelError):
        read_filterbank(p)
    with pytest.raises(AccelError):
        read_filterbank(tmp_path / "missing.fil")
