"""Shared helpers for the test suite (host-side synthetic inputs, comparisons)."""
from __future__ import annotations

import numpy as np


def synth_samples(W, H, S, G=7, seed=0, region=4, mean_mu=-1.0, mean_sigma=1.0, noise_sigma=0.5,
                  firefly_prob=1e-3, firefly_scale=1e3, zero_prob=0.0):
    """Seeded sample planes [S, 5+G, H, W] float32: per-region lognormal radiance
    means times per-sample lognormal(0, noise_sigma) noise with fireflies, uniform
    in-pixel offsets, features piecewise constant per region plus a small jitter."""
    rng = np.random.default_rng(seed)
    ry, rx = (H + region - 1) // region, (W + region - 1) // region
    mu_r = np.exp(mean_mu + mean_sigma * rng.standard_normal((3, ry, rx)))
    f_r = rng.random((G, ry, rx))
    yy, xx = np.meshgrid(np.arange(H) // region, np.arange(W) // region, indexing="ij")
    mu = mu_r[:, yy, xx]
    fb = f_r[:, yy, xx]
    out = np.empty((S, 5 + G, H, W), np.float32)
    noise = np.exp(noise_sigma * rng.standard_normal((S, 3, H, W)))
    ff = np.where(rng.random((S, 1, H, W)) < firefly_prob, firefly_scale, 1.0)
    rad = mu[None] * noise * ff
    if zero_prob > 0:
        rad = np.where(rng.random((S, 1, H, W)) < zero_prob, 0.0, rad)
    out[:, 0:3] = rad
    out[:, 3:5] = rng.random((S, 2, H, W))
    out[:, 5:] = np.clip(fb[None] + 0.02 * (rng.random((S, G, H, W)) - 0.5), 0.0, 1.0)
    return out


def rel_err(a, b, floor):
    """max |a-b| / max(|b|, floor) with a per-element floor array or scalar."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def moment_scale(stats, n, q):
    """Natural magnitude of moment q (1-based power) per element: n * s^q with s
    the per-pixel standard deviation, used as the absolute floor of relative
    errors (central moments near zero would otherwise divide by ~0)."""
    m2 = np.abs(stats[:, 1])
    nn = np.maximum(n, 1)[None, None]
    s = np.sqrt(m2 / nn)
    return nn * s ** q + 1e-300
