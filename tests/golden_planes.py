"""Access to tests/golden/reference_planes.npz (written by
tests/golden/make_plane_golden.py from the reference's own host code and
kernel source): per case and step, the whitened input rebuilt from the bins
the step reads, and the reference's fundamental powers and stage sums over
a window of columns."""
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_planes.npz")


def load():
    return dict(np.load(PATH))


def cases(g):
    """[(case, step, zmax, numharm, uselen, numbins, startr, window, stages)]"""
    out = []
    for k in sorted(g):
        if not k.endswith("_startr"):
            continue
        key = k[: -len("_startr")]
        case, step = key.split("_s")
        zmax, numharm, uselen, n, numbins, rlo = (int(v) for v in g[case + "_meta"])
        out.append((case, int(step), zmax, numharm, uselen, numbins, int(g[k][0]),
                    tuple(int(v) for v in g[key + "_window"]), g[key + "_stages"]))
    return out


def spectrum(g, case, step, numbins):
    """The whitened spectrum with the step's bins filled in (zeros elsewhere:
    no stage of the step reads them)."""
    key = f"{case}_s{step}"
    w = np.zeros(numbins, np.complex64)
    bins = g[key + "_bins"]
    o = 0
    for a, b in g[key + "_ranges"]:
        w[a:b] = bins[o: o + (b - a)]
        o += b - a
    assert o == bins.size
    return w
