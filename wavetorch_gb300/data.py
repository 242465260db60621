"""Synthetic stand-ins for the reference's vowel recordings.

The reference trains on Hillenbrand vowel recordings resampled to 10 kHz
(wavetorch/data/vowels.py:20-99).  These are not shipped or reproduced here;
the workloads use seeded formant-like waveforms of the same length, sample
rate and peak normalisation instead.
"""
from __future__ import annotations

import numpy as np

SAMPLE_RATE = 10_000.0
FORMANT_BANDS = ((300.0, 800.0), (800.0, 2500.0), (2000.0, 3500.0))


def vowel_like(batch: int, steps: int, seed: int = 0, n_classes: int = 3):
    """Return (x [batch, steps] float32, labels [batch] int64).

    x_b(t) = hann(t) * sum_k a_k sin(2 pi f_k t / 10 kHz + phi_k), with
    f_k ~ U(band_k), a_k ~ U(0.2, 1), phi_k ~ U(0, 2 pi), scaled to max |x| = 1;
    labels ~ U{0 .. n_classes-1}."""
    rng = np.random.default_rng(seed)
    t = np.arange(steps, dtype=np.float64)
    hann = np.hanning(steps) if steps > 1 else np.ones(1)
    x = np.zeros((batch, steps), dtype=np.float64)
    for k in range(batch):
        s = np.zeros(steps)
        for lo, hi in FORMANT_BANDS:
            f = rng.uniform(lo, hi)
            a = rng.uniform(0.2, 1.0)
            phi = rng.uniform(0.0, 2 * np.pi)
            s += a * np.sin(2 * np.pi * f * t / SAMPLE_RATE + phi)
        s *= hann
        m = np.abs(s).max()
        x[k] = s / m if m > 0 else s
    labels = rng.integers(0, n_classes, size=batch)
    return x.astype(np.float32), labels.astype(np.int64)


def sinusoid(steps: int, cycles_per_step: float, amplitude: float = 1.0):
    """x_t = amplitude * sin(2 pi f t), t = 0 .. steps-1 (float32, [1, steps])."""
    t = np.arange(steps, dtype=np.float64)
    return (amplitude * np.sin(2 * np.pi * cycles_per_step * t)).astype(np.float32)[None, :]
