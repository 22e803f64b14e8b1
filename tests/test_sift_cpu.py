"""Candidate sifting (accel_sift_candidates, host only) against its plain
restatement in the oracle: same survivors in the same order, on seeded
candidate lists with clusters of threshold crossings, harmonically related
signals and noise, over several trials.  No GPU needed."""
import numpy as np
import pytest

import __graft_entry__
from gpu_accelsearch_gb300.search import CAND_DTYPE, sift_candidates
from oracle import oracle as O


@pytest.fixture(scope="module", autouse=True)
def lib():
    __graft_entry__.build_library()


def make_cands(seed, ntrials=2):
    rng = np.random.default_rng(seed)
    rows = []
    for t in range(ntrials):
        for _ in range(4):  # signals: a cluster, and weaker clusters at harmonics of it
            r0 = rng.uniform(2e4, 2e5)
            z0 = rng.uniform(-100, 100)
            for ratio, scale in [(1.0, 1.0), (2.0, 0.6), (1.5, 0.5), (0.5, 0.55), (4 / 3, 0.4)]:
                for _ in range(rng.integers(5, 40)):
                    r = r0 * ratio + rng.normal(0, 3)
                    sig = scale * rng.uniform(8, 20) - abs(r - r0 * ratio) * 0.05
                    rows.append((t, rng.integers(0, 500), round(2 * r) / 2, z0 + rng.normal(0, 4),
                                 int(rng.choice([1, 2, 4, 8])), sig * 3, sig))
        for _ in range(150):  # noise crossings
            r = rng.uniform(1e3, 3e5)
            sig = rng.uniform(6, 7)
            rows.append((t, rng.integers(0, 500), round(2 * r) / 2, 2 * rng.integers(-100, 101),
                         int(rng.choice([1, 2, 4, 8])), sig * 3, sig))
    a = np.array(rows, dtype=CAND_DTYPE)
    return a[rng.permutation(len(a))]


def key(c):
    return (int(c["trial"]), float(c["r"]), float(c["z"]), int(c["numharm"]), float(c["sigma"]))


@pytest.mark.parametrize("seed,min_dr,maxharm,harm_dr", [(1, 15.0, 8, 1.0), (2, 15.0, 16, 2.0),
                                                          (3, 5.0, 1, 1.0), (4, 0.0, 8, 0.5),
                                                          (5, 30.0, 4, 1.0)])
def test_sift_matches_oracle(seed, min_dr, maxharm, harm_dr):
    c = make_cands(seed)
    got = sift_candidates(c, min_dr=min_dr, maxharm=maxharm, harm_dr=harm_dr)
    want = O.sift(c, min_dr=min_dr, maxharm=maxharm, harm_dr=harm_dr)
    assert [key(x) for x in got] == [key(x) for x in want]
    assert 0 < len(got) < len(c)


def test_sift_keeps_one_per_signal():
    # one strong cluster and its 2nd harmonic in one trial: one survivor each
    # without harmonic elimination, one in total with it
    rng = np.random.default_rng(9)
    rows = [(0, 0, 50000.0 + d, 10.0, 1, 90.0 - abs(d), 30.0 - abs(d) / 3) for d in np.arange(-8, 8.5, 0.5)]
    rows += [(0, 0, 100000.0 + d, 20.0, 2, 60.0 - abs(d), 20.0 - abs(d) / 3) for d in np.arange(-8, 8.5, 0.5)]
    c = np.array(rows, dtype=CAND_DTYPE)[rng.permutation(len(rows))]
    one = sift_candidates(c, min_dr=15.0, maxharm=1)
    assert sorted(float(x["r"]) for x in one) == [50000.0, 100000.0]
    both = sift_candidates(c, min_dr=15.0, maxharm=8, harm_dr=1.0)
    assert [float(x["r"]) for x in both] == [50000.0]


def test_sift_rejects_bad_arguments():
    from gpu_accelsearch_gb300 import native as N
    c = make_cands(1, 1)
    with pytest.raises(N.AccelError):
        sift_candidates(c, min_dr=-1.0)
    with pytest.raises(N.AccelError):
        sift_candidates(c, maxharm=0)
    assert len(sift_candidates(c[:0])) == 0
