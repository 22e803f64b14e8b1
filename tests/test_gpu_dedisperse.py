"""Dedispersion on the GPU against the oracle's direct sum (bit-exact: the
same float32 additions in channel order), and a dispersed periodic signal
recovered by the batched search at its DM trial."""
import numpy as np
import pytest

from gpu_accelsearch_gb300.dedisperse import dedisperse, dm_delays
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


# the windowed kernel (channel windows in shared memory, 16 trials per CTA:
# trial counts below, at and above a tile, channel counts that are not a
# multiple of its 8-channel chunks, output lengths that end inside a tile),
# and the one-load-per-addition kernel it falls back to when a tile's
# delays spread too far for its windows (coarse DM steps: the first, third
# and last two cases)
@pytest.mark.parametrize("nchan,nsamp,dms", [(64, 30000, np.arange(0, 130, 10)),
                                             (7, 5000, [0.0, 3.5]),
                                             (200, 9000, np.arange(0, 40, 2.5)),
                                             (1027, 12000, np.arange(0, 33, 1.0)),
                                             (256, 70000, np.arange(0, 64, 1.0)),
                                             (64, 30000, np.arange(0, 20, 0.5)),
                                             (96, 70000, np.arange(0, 1601, 100.0)),
                                             (48, 400000, np.arange(0, 7001, 500.0))])
def test_dedisperse_bit_exact(nchan, nsamp, dms):
    rng = np.random.default_rng(nchan)
    fb = rng.standard_normal((nchan, nsamp)).astype(np.float32)
    dl, mx = dm_delays(nchan, 1400.0, -300.0 / nchan, 64e-6, dms)
    nout = nsamp - mx - 3
    d_fb = torch.from_numpy(fb).cuda()
    d_out = torch.full((len(dms), nout), np.nan, dtype=torch.float32, device="cuda")
    dedisperse(d_fb.data_ptr(), nchan, nsamp, dl, d_out.data_ptr(), nout)
    torch.cuda.synchronize()
    got = d_out.cpu().numpy()
    want = O.dedisperse(fb, dl, nout)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_too_few_samples_rejected():
    from gpu_accelsearch_gb300.native import AccelError
    dl, mx = dm_delays(8, 1400.0, -10.0, 64e-6, [0.0, 50.0])
    d_fb = torch.zeros((8, 1000), dtype=torch.float32, device="cuda")
    d_out = torch.zeros((2, 1000), dtype=torch.float32, device="cuda")
    with pytest.raises(AccelError):
        dedisperse(d_fb.data_ptr(), 8, 1000, dl, d_out.data_ptr(), 1000 - mx + 1)


def test_dispersed_signal_found_at_its_dm():
    # a periodic signal dispersed at DM 30 in 64 channels (1400 MHz top, 300 MHz
    # band) plus independent noise per channel; dedispersed at DM 0..60 and all
    # trials searched in one batched call: the signal is strongest in trial 3
    from gpu_accelsearch_gb300.search import AccelSearch
    nchan, n, dt = 64, 1 << 18, 64e-6
    dms = np.arange(0, 61, 10, dtype=np.float32)
    dl, mx = dm_delays(nchan, 1400.0, -300.0 / nchan, dt, dms)
    true = dl[3]
    nsamp = n + mx
    rng = np.random.default_rng(11)
    t = np.arange(nsamp, dtype=np.float64)
    r0 = 20000.25
    fb = rng.standard_normal((nchan, nsamp)).astype(np.float32)
    for c in range(nchan):  # channel c sees the signal true[c] samples late
        fb[c] += (0.03 * np.cos(2 * np.pi * r0 * (t - true[c]) / n)).astype(np.float32)
    d_fb = torch.from_numpy(fb).cuda()
    d_out = torch.empty((len(dms), n), dtype=torch.float32, device="cuda")
    dedisperse(d_fb.data_ptr(), nchan, nsamp, dl, d_out.data_ptr(), n)
    ptrs = [d_out[i].data_ptr() for i in range(len(dms))]
    with AccelSearch(zmax=50, numharm=4, fftlen=2048) as s:
        s.search(ptrs, dt, on_device=True, nsamples=[n] * len(dms))
        c = s.candidates()
    near = c[(np.abs(c["r"] - r0) <= 1.0) & (np.abs(c["z"]) <= 2.0) & (c["numharm"] == 1)]
    assert len(near) > 0
    best = near[np.argmax(near["power"])]
    assert int(best["trial"]) == 3
