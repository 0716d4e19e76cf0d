"""Seeded synthetic MEMD inputs in numpy (no compiled code).

The benchmark (both of its arms) and the full-size parity fixtures draw their
records from here, so that a process that must not load the CUDA library (the
CPU baseline arm) still decomposes exactly the record the GPU arm does.  The
C++ generator exported by libmemd_gb300.so (memd_synth_eeg / memd_synth_tones)
draws from the same signal families with a different random stream.

eeg(C, L, fs, seed)    C independent 1/f (pink) sources mixed by a seeded
                       C x C Gaussian matrix, plus 10 Hz alpha bursts
                       (Hann-windowed, 1-3 s, Poisson arrivals at 0.2/s) and a
                       0.5 Hz drift, scaled to tens of units (EEG-like).
tones(C, L, fs, seed)  tones at 5, 20 and 60 Hz with per-channel amplitudes
                       U[0.5, 1.5] and phases U[0, 2 pi), plus N(0, 0.1^2)
                       noise.
"""
from __future__ import annotations

import numpy as np

_PINK_SECTIONS = 14


def _pink(rng: np.random.Generator, C: int, L: int, fs: float) -> np.ndarray:
    """1/f noise: white noise through one-pole low-pass sections
    y[n] = a y[n-1] + (1 - a) x[n] with corners spaced by a factor 2 from fs/4
    down, weighted by 1/sqrt(corner) (unit gain below each corner, so the
    summed power density is close to 1/f across the band).  The filters run
    for three time constants of the slowest section before the record starts."""
    from scipy.signal import lfilter

    f = fs / 4.0 * 0.5 ** np.arange(_PINK_SECTIONS)
    a = np.exp(-2.0 * np.pi * f / fs)
    w = 1.0 / np.sqrt(f)
    tau = fs / (2.0 * np.pi * f[-1])
    nwarm = int(min(3.0 * tau, 200000.0))
    x = rng.standard_normal((C, nwarm + L))
    out = np.zeros((C, nwarm + L))
    for j in range(_PINK_SECTIONS):
        out += w[j] * lfilter([1.0 - a[j]], [1.0, -a[j]], x, axis=1)
    return out[:, nwarm:]


def eeg(C: int, L: int, fs: float = 256.0, seed: int = 0) -> np.ndarray:
    """C x L float64 EEG-shaped record (channel-major)."""
    rng = np.random.default_rng([0x4D454D44, int(seed)])
    src = _pink(rng, C, L, fs)
    src /= np.sqrt(np.mean(src * src, axis=1, keepdims=True))
    mix = rng.standard_normal((C, C)) / np.sqrt(C)
    out = mix @ src
    gain = 1.5 * rng.standard_normal(C)
    t, dur = 0.0, L / fs
    while True:
        t += rng.exponential(1.0 / 0.2)
        if t >= dur:
            break
        d = rng.uniform(1.0, 3.0)
        ph = rng.uniform(0.0, 2.0 * np.pi)
        n0, nd = int(t * fs), int(d * fs)
        k = np.arange(min(nd, L - n0))
        v = (0.5 - 0.5 * np.cos(2.0 * np.pi * k / nd)) * np.sin(2.0 * np.pi * 10.0 * k / fs + ph)
        out[:, n0:n0 + k.size] += gain[:, None] * v[None, :]
    amp = rng.uniform(0.5, 1.5, C)
    ph = rng.uniform(0.0, 2.0 * np.pi, C)
    n = np.arange(L)
    out = 30.0 * (out + amp[:, None] * np.sin(2.0 * np.pi * 0.5 * n[None, :] / fs + ph[:, None]))
    return np.ascontiguousarray(out)


def tones(C: int, L: int, fs: float = 1000.0, seed: int = 0) -> np.ndarray:
    """C x L float64 three-tone mixture with white noise (channel-major)."""
    rng = np.random.default_rng([0x544F4E45, int(seed)])
    n = np.arange(L) / fs
    amp = rng.uniform(0.5, 1.5, (C, 3))
    ph = rng.uniform(0.0, 2.0 * np.pi, (C, 3))
    out = np.zeros((C, L))
    for j, fr in enumerate((5.0, 20.0, 60.0)):
        out += amp[:, j:j + 1] * np.sin(2.0 * np.pi * fr * n[None, :] + ph[:, j:j + 1])
    out += 0.1 * rng.standard_normal((C, L))
    return np.ascontiguousarray(out)


def as_float32_record(y: np.ndarray) -> np.ndarray:
    """The record rounded to float32 once and widened back exactly, so that
    the FP64 and the float32-input forms decompose the same numbers."""
    return np.ascontiguousarray(y, dtype=np.float32).astype(np.float64)
