"""Candidate keys shared by the parity tests: (step, r index, z index,
numharm) from either the library's candidates (r, z in bins) or the
oracle's (indices), and the oracle's candidate sets just inside and just
outside a +-tol relative band around each stage cut."""
import numpy as np


def keys(a, rlo=0, half=0, zlo0=0):
    if "ridx" in a.dtype.names:
        return {(int(c["step"]), int(c["ridx"]), int(c["zidx"]), int(c["numharm"])) for c in a}
    return {(int(c["step"]), int(round(2 * (c["r"] - (rlo + c["step"] * half)))),
             int(round((c["z"] - zlo0) / 2)), int(c["numharm"])) for c in a}


def oracle_bounds(orc, wspec, rlo, step0, nsteps, cuts, tol=1e-4, cap=1 << 22):
    """(keys above cut*(1+tol), keys above cut*(1-tol)) of the FP64 oracle:
    a GPU candidate set equal to the oracle's outside the band lies between."""
    c = np.asarray(cuts, np.float64)
    hi, _, nhi = orc.run_steps(wspec, rlo, step0, nsteps, powcut=c * (1 + tol), cap=cap)
    lo, _, nlo = orc.run_steps(wspec, rlo, step0, nsteps, powcut=c * (1 - tol), cap=cap)
    assert nlo <= cap and nhi <= cap
    return keys(hi), keys(lo)
