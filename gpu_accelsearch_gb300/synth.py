"""Seeded synthetic DM-trial time series (host side, numpy).

No public dataset is involved: the reference reads a raw float32 ``.dat``
time series (bpd_data.c:9-75).  These generators stand in for it with
N(0,1) noise plus optional accelerated sinusoids
x[n] += A cos(2 pi (r0 t + z t^2 / 2)), t = n/N, where r0 is the Fourier
frequency in bins and z the f-dot in bins (drift over the observation).
"""
from __future__ import annotations

import numpy as np


def synth_series(n: int, seed: int, signals=()) -> np.ndarray:
    """float32[n]: N(0,1) noise (PCG64) plus (amplitude, r0, z) sinusoids."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n, dtype=np.float32)
    if signals:
        t = np.arange(n, dtype=np.float64) / n
        acc = np.zeros(n, np.float64)
        for amp, r0, z in signals:
            acc += amp * np.cos(2.0 * np.pi * (r0 * t + 0.5 * z * t * t))
        x = (x.astype(np.float64) + acc).astype(np.float32)
    return x


def synth_red_spectrum(numbins: int, seed: int) -> np.ndarray:
    """complex64[numbins]: Gaussian spectrum with a red-noise envelope."""
    rng = np.random.default_rng(seed)
    re = rng.standard_normal(numbins, dtype=np.float32)
    im = rng.standard_normal(numbins, dtype=np.float32)
    k = np.arange(numbins, dtype=np.float64)
    env = (1.0 + 20.0 / np.sqrt(1.0 + k / 30.0)).astype(np.float32)
    return ((re * env) + 1j * (im * env)).astype(np.complex64)
