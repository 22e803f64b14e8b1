"""The continuous-batching request server (accel_server_*) on the GPU."""
import time

import numpy as np
import pytest

from gpu_accelsearch_gb300.synth import synth_series

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
DT = 64e-6
FIELDS = ["step", "r", "z", "numharm", "power", "sigma"]


def same(a, b):
    return len(a) == len(b) and all(np.array_equal(a[f], b[f]) for f in FIELDS)


def test_alone_equals_mixed_and_context_path():
    from gpu_accelsearch_gb300.search import AccelSearch
    from gpu_accelsearch_gb300.serving import Server
    a = synth_series(1 << 18, seed=1, signals=[(0.05, 20000.25, 40.0)])
    others = [(synth_series(1 << 17, seed=2, signals=[(0.1, 9000.5, -30.0)]), 100),
              (synth_series(1 << 18, seed=3), 50),
              (synth_series(1 << 16, seed=4, signals=[(0.2, 3000.0, 10.0)]), 200)]
    with Server(hbm_budget_bytes=2e9, fftlen=2048, numharm=4, chunk_segments=16) as srv:
        rid = srv.submit(a, DT, 50)
        assert srv.wait(rid, 60)
        alone, _ = srv.result(rid)
        ids = [srv.submit(x, DT, z) for x, z in others[:2]]
        rid2 = srv.submit(a, DT, 50)
        ids.append(srv.submit(*others[2][:1], DT, others[2][1]))
        for i in ids + [rid2]:
            assert srv.wait(i, 60)
        mixed, _ = srv.result(rid2)
        st = srv.stats()
        assert st["completed"] == 5 and st["active"] == 0 and st["bytes_in_use"] == 0
    assert len(alone) > 0
    assert same(alone, mixed)
    with AccelSearch(zmax=50, numharm=4, fftlen=2048) as s:
        s.search([a], DT)
        assert same(alone, s.candidates())


def test_budget_admission_and_rejection():
    from gpu_accelsearch_gb300.native import AccelError
    from gpu_accelsearch_gb300.serving import Server
    n = 1 << 17
    per = 4.0 * n + 8.0 * (n // 2 + 1)
    with Server(hbm_budget_bytes=2.5 * per, fftlen=2048, numharm=4, chunk_segments=8) as srv:
        xs = [synth_series(n, seed=10 + i) for i in range(5)]
        ids = [srv.submit(x, DT, 50) for x in xs]
        for i in ids:
            assert srv.wait(i, 60)
        st = srv.stats()
        assert st["completed"] == 5 and st["bytes_in_use"] == 0
        with pytest.raises(AccelError) as e:
            srv.submit(synth_series(1 << 19, seed=99), DT, 50)
        assert e.value.code == -6


def test_continuous_batching_short_request_overtakes():
    from gpu_accelsearch_gb300.serving import Server
    long_x = synth_series(1 << 23, seed=20)
    short_x = synth_series(1 << 15, seed=21)
    with Server(hbm_budget_bytes=4e9, fftlen=2048, numharm=4, chunk_segments=16) as srv:
        assert srv.wait(srv.submit(short_x, DT, 50), 60)  # bank built before the measurement
        lid = srv.submit(long_x, DT, 50)
        while srv.stats()["active"] == 0:  # wait until the long request is being searched
            time.sleep(0.001)
        sid = srv.submit(short_x, DT, 50)
        long_running = not srv.wait(lid, 0.0)
        assert srv.wait(sid, 60)
        short_done_first = not srv.wait(lid, 0.0)
        assert srv.wait(lid, 300)
        _, lat_long = srv.result(lid)
        _, lat_short = srv.result(sid)
        parts = [srv.timing(lid), srv.timing(sid)]
        st = srv.stats()
    assert long_running and short_done_first
    assert lat_short < lat_long
    # the latency breakdown adds up to the latency, every part non-negative
    for lat, p in zip((lat_long, lat_short), parts):
        assert all(v >= 0 for v in p.values()), p
        assert abs(sum(p.values()) - lat) < 1e-6 * lat + 1e-3, (p, lat)
    assert st["gap_ms"] >= 0 and st["idle_ms"] >= 0
    # the scheduler's launch and wait time are parts of its group time; every
    # launch group read back is counted with its segments
    assert 0 <= st["launch_ms"] <= st["group_ms"] and 0 <= st["wait_ms"] <= st["group_ms"]
    assert st["groups"] > 0 and st["group_segments"] >= st["groups"] and st["prep_gpu_ms"] > 0


@pytest.mark.parametrize("max_chunk", [0, 64])
def test_many_lengths_and_banks_equal_context_path(max_chunk):
    # every request a new series length (odd factors of every size: the
    # transform's power-of-two, Cooley-Tukey and Bluestein forms), two
    # banks, submitted at once; with max_chunk the launch groups grow with
    # the backlog (16 to 64 segments)
    from gpu_accelsearch_gb300.search import AccelSearch
    from gpu_accelsearch_gb300.serving import Server
    rng = np.random.default_rng(77)
    reqs = []
    for i in range(12):
        n = 2 * int(rng.integers(1 << 14, 1 << 16))
        z = 50 if i % 3 else 100
        reqs.append((synth_series(n, seed=300 + i, signals=[(0.1, 0.2 * n + 0.25, 8.0)]), z))
    with Server(hbm_budget_bytes=4e9, fftlen=2048, numharm=4, chunk_segments=16,
                max_chunk_segments=max_chunk) as srv:
        ids = [srv.submit(x, DT, z) for x, z in reqs]
        for i in ids:
            assert srv.wait(i, 120)
        got = [srv.result(i)[0] for i in ids]
        assert srv.stats()["completed"] == len(reqs)
    for (x, z), g in zip(reqs, got):
        with AccelSearch(zmax=z, numharm=4, fftlen=2048) as s:
            s.search([x], DT)
            assert same(g, s.candidates()), (x.size, z)


def test_wait_limit_bounds_a_long_request_under_a_flood_of_short_ones():
    # 600 short requests queued behind one long request: shortest remaining
    # work first alone would serve every short one first (~1.5 s of GPU
    # work); with max_wait_s = 0.3 the long request gets every other launch
    # group once it has waited 0.3 s, while short ones still overtake it
    # before that
    from gpu_accelsearch_gb300.serving import Server
    long_x = synth_series(1 << 23, seed=30)
    short_x = synth_series(1 << 20, seed=31)
    with Server(hbm_budget_bytes=40e9, fftlen=8192, numharm=8, chunk_segments=128, max_wait_s=0.3) as srv:
        assert srv.wait(srv.submit(short_x, DT, 200), 120)  # bank built before the measurement
        lid = srv.submit(long_x, DT, 200)
        sids = [srv.submit(short_x, DT, 200) for _ in range(600)]
        assert srv.wait(lid, 300)
        short_done_before = sum(1 for i in sids if srv.wait(i, 0.0))
        for i in sids:
            assert srv.wait(i, 300)
        _, lat_long = srv.result(lid)
        lat_short = [srv.result(i)[1] for i in sids]
    assert short_done_before > 0          # shorter work still went first
    assert short_done_before < len(sids)  # but not all of it: the wait limit cut in
    assert lat_long < 0.3e3 + 0.7e3, lat_long  # limit + its own search and group latency
    assert max(lat_short) > lat_long
